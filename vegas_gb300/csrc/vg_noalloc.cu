// vg_noalloc.cu -- a vegas+ iteration that allocates no device memory.
//
// vg_iteration_noalloc runs the same kernels as vg_allocate +
// vg_fused_iteration + vg_end_iteration, but its scratch space is a
// file-scope device array instead of a caller-provided workspace.  It exists
// for callers that cannot allocate device memory themselves: a plug-in whose
// host application owns every device byte through its own pool allocator, a
// service running under a hard device-memory budget, or a caller that must
// not allocate on its iteration path.  Such callers still pass the
// integrator's grid, sigf, training histogram and stats record (its inputs
// and outputs); only the scratch lives here.
//
// The array (VG_NOALLOC_SCRATCH_BYTES) is reserved on every GPU that loads
// this library, for the life of the process.
#include <mutex>
#include <string.h>

#include "vg_common.cuh"

static __device__ __align__(256) unsigned char g_vg_noalloc_scratch[VG_NOALLOC_SCRATCH_BYTES];

int vg_alloc_sync_reset(const vg_integrator *it, void *stream);   // vg_iter.cu

namespace {
std::mutex g_mutex;
void *g_scratch[VG_MAX_DEVICES];   // device address of the array, per device ordinal
}  // namespace

// Device address of the scratch array for the current device.  The first
// call on a device looks it up with cudaGetSymbolAddress (the host-side name
// of the array is only a stand-in, never a device address).  The cached
// address assumes the device's primary context stays alive: after a
// cudaDeviceReset the module is loaded again and the address may change.
static int scratch_address(void **out)
{
    int dev = 0;
    VG_CUDA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= VG_MAX_DEVICES) return vg_fail(VG_ERR_UNSUPPORTED, "device ordinal %d", dev);
    std::lock_guard<std::mutex> lock(g_mutex);
    if (g_scratch[dev] == nullptr) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_vg_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr)
            return vg_fail(VG_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
        g_scratch[dev] = p;
    }
    *out = g_scratch[dev];
    return VG_OK;
}

extern "C" int vg_iteration_noalloc(const vg_integrator *it, uint32_t itn, const double *u, int kind,
                                    const double *params, int nparams, void *stream)
{
    VG_RANGE("vg_iteration_noalloc");
    vg_clear_error();
    if (it == nullptr) return vg_fail(VG_ERR_VALUE, "vg_iteration_noalloc: no integrator");
    if (it->dim < 1 || it->dim > VG_MAX_DIM)   // before anything reads ninc[0 .. dim)
        return vg_fail(VG_ERR_VALUE, "vg_iteration_noalloc: dim %d outside 1..%d", it->dim, VG_MAX_DIM);
    void *scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return rc;
    vg_integrator local;
    memcpy(&local, it, sizeof(local));
    local.work = nullptr;
    local.work_bytes = 0;
    const size_t need = vg_workspace_bytes(&local, 0);
    if (need > (size_t)VG_NOALLOC_SCRATCH_BYTES)
        return vg_fail(VG_ERR_MEMORY,
                       "vg_iteration_noalloc: this iteration needs %zu bytes of scratch, above the "
                       "%d-byte static limit; use vg_allocate/vg_fused_iteration with a workspace",
                       need, VG_NOALLOC_SCRATCH_BYTES);
    local.work = scratch;
    local.work_bytes = (size_t)VG_NOALLOC_SCRATCH_BYTES;
    // the scratch is shared by every geometry: start the allocation's
    // published words afresh
    if ((rc = vg_alloc_sync_reset(&local, stream))) return rc;
    if ((rc = vg_allocate(&local, stream))) return rc;
    if ((rc = vg_fused_iteration(&local, itn, u, kind, params, nparams, stream))) return rc;
    return vg_end_iteration(&local, stream);
}
