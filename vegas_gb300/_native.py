"""Build and load ``libvegas_gb300.so`` (the C ABI in include/vegas_gb300.h).

The library is compiled in-tree (``vegas_gb300/_native/``) from
``vegas_gb300/csrc``: the CUDA files with nvcc for sm_103a only, the host
C file with gcc.  It is bound with ctypes: there are no torch types in the
ABI; tensors are passed as raw device pointers plus the current CUDA stream.

There is no CPU fallback: if the library cannot be built or loaded, or no
CUDA device is present, every device operation raises.
"""
import ctypes
import glob
import os
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
OUT = os.path.join(HERE, '_native')
LIBNAME = 'libvegas_gb300.so'
LIBPATH = os.path.join(OUT, LIBNAME)
INCLUDE = os.path.join(os.path.dirname(HERE), 'include')

ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
NVCC_FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '--expt-relaxed-constexpr']

VG_MAX_DIM = 64
VG_NOALLOC_SCRATCH_BYTES = 16 * 1024 * 1024
VG_BATCH_CFG_F64 = 16
VG_F32, VG_F64 = 0, 1
VG_OK, VG_ERR_VALUE, VG_ERR_MEMORY, VG_ERR_CUDA, VG_ERR_NAN, VG_ERR_UNSUPPORTED, VG_ERR_TIMEOUT = range(7)
(VG_F_GAUSS, VG_F_RIDGE, VG_F_LORENTZ, VG_F_MIXTURE, VG_F_LATTICE, VG_F_CONST) = range(6)


def _nvcc():
    for c in (os.environ.get('NVCC'), '/usr/local/cuda/bin/nvcc', 'nvcc'):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return 'nvcc'


def _sources():
    cu = sorted(glob.glob(os.path.join(CSRC, '*.cu')))
    c = sorted(glob.glob(os.path.join(CSRC, '*.c')))
    hdr = sorted(glob.glob(os.path.join(CSRC, '*.h')) + glob.glob(os.path.join(CSRC, '*.cuh'))
                 + glob.glob(os.path.join(INCLUDE, '*.h')))
    return cu, c, hdr


def _stale():
    if not os.path.exists(LIBPATH):
        return True
    t = os.path.getmtime(LIBPATH)
    cu, c, hdr = _sources()
    return any(os.path.getmtime(f) > t for f in cu + c + hdr)


def build(force=False, verbose=False):
    """Compile every CUDA/C source for sm_103a and link the shared library."""
    if not force and not _stale():
        return LIBPATH
    os.makedirs(OUT, exist_ok=True)
    cu, c, _ = _sources()
    nvcc = _nvcc()
    objs = []
    cmds = []
    for f in cu:
        o = os.path.join(OUT, os.path.basename(f) + '.o')
        objs.append(o)
        cmds.append([nvcc] + ARCH + NVCC_FLAGS + ['-I', CSRC, '-I', INCLUDE, '-c', f, '-o', o])
    for f in c:
        o = os.path.join(OUT, os.path.basename(f) + '.o')
        objs.append(o)
        cmds.append(['gcc', '-std=gnu11', '-O2', '-ffp-contract=off', '-fPIC', '-Wall',
                     '-I', CSRC, '-I', INCLUDE, '-c', f, '-o', o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('build failed: %s\n%s%s' % (' '.join(cmd), r.stdout, r.stderr))
        if verbose:
            print(' '.join(cmd))
        return r

    with ThreadPoolExecutor(max_workers=max(2, min(len(cmds), os.cpu_count() or 4))) as ex:
        list(ex.map(run, cmds))
    tmp = LIBPATH + '.%d.tmp' % os.getpid()
    run([nvcc] + ARCH + ['-shared', '-o', tmp] + objs + ['-lm', '-ldl'])
    os.replace(tmp, LIBPATH)
    return LIBPATH


class VgStats(ctypes.Structure):
    _fields_ = [
        ('sum_sigf', ctypes.c_double), ('mean', ctypes.c_double), ('var', ctypes.c_double),
        ('neval_sigf', ctypes.c_double), ('neval', ctypes.c_int64), ('range_lo', ctypes.c_int64),
        ('range_hi', ctypes.c_int64), ('ntiles', ctypes.c_int64), ('nan_seen', ctypes.c_int32),
        ('sigf_reset', ctypes.c_int32), ('status', ctypes.c_int32), ('pad', ctypes.c_int32),
    ]


class VgIntegrator(ctypes.Structure):
    _fields_ = [
        ('dim', ctypes.c_int32), ('precision', ctypes.c_int32), ('nhcube', ctypes.c_int64),
        ('nstrat', ctypes.c_int64 * VG_MAX_DIM), ('ninc', ctypes.c_int64 * VG_MAX_DIM),
        ('grid', ctypes.c_void_p), ('inc', ctypes.c_void_p), ('ldg', ctypes.c_int64),
        ('ldi', ctypes.c_int64), ('sigf', ctypes.c_void_p), ('sum_f', ctypes.c_void_p),
        ('n_f', ctypes.c_void_p), ('stats', ctypes.c_void_p), ('work', ctypes.c_void_p),
        ('work_bytes', ctypes.c_size_t), ('neval', ctypes.c_int64),
        ('neval_frac', ctypes.c_double), ('min_neval_hcube', ctypes.c_int64),
        ('max_neval_hcube', ctypes.c_int64), ('alpha', ctypes.c_double),
        ('beta', ctypes.c_double), ('adapt', ctypes.c_int32), ('adapt_to_errors', ctypes.c_int32),
        ('seed', ctypes.c_uint64), ('stream_id', ctypes.c_uint32), ('tile', ctypes.c_int32),
    ]


class VgFlow(ctypes.Structure):
    _fields_ = [
        ('dim', ctypes.c_int32), ('nlayers', ctypes.c_int32), ('K', ctypes.c_int32),
        ('hidden', ctypes.c_int32), ('theta', ctypes.c_void_p), ('mirror', ctypes.c_void_p),
        ('grad', ctypes.c_void_p), ('adam_m', ctypes.c_void_p), ('adam_v', ctypes.c_void_p),
        ('loss', ctypes.c_void_p),
    ]


_lock = threading.Lock()
_lib = None

# every exported symbol and its signature (restype, argtypes)
P, I32, I64, U32, U64, DBL, SZ = (ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_uint32,
                                  ctypes.c_uint64, ctypes.c_double, ctypes.c_size_t)
SIGNATURES = {
    'vg_last_error': (ctypes.c_char_p, []),
    'vg_version': (I32, []),
    'vg_struct_size': (SZ, [I32]),
    'vg_set_strata': (I32, [I32, I32, P, I32, P, DBL, DBL, I32, I32, DBL, I32, I64, P, P, P]),
    'vg_neval_cap': (I64, [P]),
    'vg_workspace_bytes': (SZ, [P, I64]),
    'vg_make_uniform': (I32, [I32, P, P, P, P, I64, P, I64, P]),
    'vg_adapt': (I32, [I32, P, P, P, P, I64, I64, P, P, DBL, P, P, I64, I64, P]),
    'vg_map': (I32, [I32, P, P, P, I64, I64, I64, P, P, P, I32, P]),
    'vg_invmap': (I32, [I32, P, P, P, I64, I64, I64, P, P, P, I32, P]),
    'vg_jac1d': (I32, [I32, P, P, I64, I64, P, P, I32, P]),
    'vg_add_training_data': (I32, [I32, P, I64, I64, P, P, I32, P, P, P]),
    'vg_allocate': (I32, [P, P]),
    'vg_stats_reset': (I32, [P, DBL, P]),
    'vg_sample': (I32, [P, U32, P, P, P, P, P, I64, P]),
    'vg_reduce': (I32, [P, U32, P, P, I32, P]),
    'vg_keep_bytes': (SZ, [P, I64]),
    'vg_sample_keep': (I32, [P, U32, P, P, P, P, P, I64, P, SZ, P]),
    'vg_reduce_kept': (I32, [P, U32, P, P, I32, P, SZ, P]),
    'vg_fused_iteration': (I32, [P, U32, P, I32, P, I32, P]),
    'vg_end_iteration': (I32, [P, P]),
    'vg_iterate': (I32, [P, U32, I32, P, I32, P]),
    'vg_reduce_array': (I32, [P, P, I32, I32, I32, P, P, P, P, SZ, P]),
    'vg_reduce_array_work_bytes': (SZ, [I32, I32]),
    'vg_iteration_noalloc': (I32, [P, U32, P, I32, P, I32, P]),
    'vg_flow_nparams': (I64, [I32, I32, I32, I32]),
    'vg_flow_mirror_elems': (I64, [I32, I32, I32, I32]),
    'vg_flow_train_bytes': (I64, [P, I64]),
    'vg_flow_refresh': (I32, [P, P]),
    'vg_flow_sample': (I32, [P, I64, P, P, P, P]),
    'vg_flow_density': (I32, [P, I64, P, P, P, P]),
    'vg_flow_grad': (I32, [P, I64, P, P, P, SZ, P]),
    'vg_flow_adam': (I32, [P, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                           ctypes.c_float, I32, ctypes.c_float, P]),
    'vg_flow_status': (I32, [P, I32]),
    'vg_flow_set_path': (I32, [I32]),
    'vg_batch_variants': (I32, []),
    'vg_batch_table_bytes': (SZ, [I32]),
    'vg_batch_prepare': (I32, [P, I32, I32, P, I32, P, I32, P, P, P, P, P, SZ, P, P, P]),
    'vg_batch_launch': (I32, [P, I32, I32, I32, I32, U32, P, P, P, P, P, P, P, P, P, P]),
    'vg_eval_points': (I32, [I32, P, I32, I32, I64, P, P, P, P, P, P, P]),
    'vg_weight_points': (I32, [I64, P, P, P, P, P]),
    'vg_flow_zero_grad': (I32, [P, P]),
    'vg_flow_train_batch': (I32, [I64, I64, U64, U32, I32, P, P, P, P, P, I32, P, P, P, P]),
    'vg_set_term_counter': (I32, [P]),
    'vg_set_eval_split': (I32, [I32]),
    'vg_set_wait_budget': (I32, [I64]),
    'vg_set_dropin_tuning': (I32, [I32, I32]),
    'vg_batch_set_stamps': (I32, [P]),
    'vg_set_tile_tuning': (I32, [I32, I32, I32]),
    'vg_probe_mufu_ex2': (I32, [P, I64, I32, P]),
    'vg_probe_fp64_fma': (I32, [P, I64, I32, P]),
    'vg_probe_fp32_fma': (I32, [P, I64, I32, P]),
    'vg_probe_umma_gemm': (I32, [P, P, P, I32, I32, I32, I32, P, P]),
}


def load(build_if_needed=True):
    """Load the library (building it first when sources are newer)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if build_if_needed:
            build()
        if not os.path.exists(LIBPATH):
            raise RuntimeError('vegas_gb300 native library missing: %s' % LIBPATH)
        L = ctypes.CDLL(LIBPATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        if (L.vg_struct_size(0) != ctypes.sizeof(VgIntegrator)
                or L.vg_struct_size(1) != ctypes.sizeof(VgStats)):
            raise RuntimeError('vegas_gb300: ctypes structure layout does not match the library')
        _lib = L
        return L


class VegasError(RuntimeError):
    pass


class VegasTimeout(VegasError):
    """A bounded device-side wait gave up (VG_ERR_TIMEOUT)."""


def check(rc):
    """Map a C-ABI status onto the exception the reference raises."""
    if rc == VG_OK:
        return
    msg = load().vg_last_error().decode(errors='replace')
    if rc == VG_ERR_VALUE or rc == VG_ERR_NAN:
        raise ValueError(msg)
    if rc == VG_ERR_MEMORY:
        raise MemoryError(msg)
    if rc == VG_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    if rc == VG_ERR_TIMEOUT:
        raise VegasTimeout('vegas_gb300 error %d: %s' % (rc, msg))
    raise VegasError('vegas_gb300 error %d: %s' % (rc, msg))


def ptr(t):
    """Raw device pointer of a torch tensor (None -> NULL)."""
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def stream_ptr(device=None):
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def i64_array(vals):
    return (ctypes.c_int64 * len(vals))(*[int(v) for v in vals])


def dbl_array(vals):
    return (ctypes.c_double * len(vals))(*[float(v) for v in vals])
