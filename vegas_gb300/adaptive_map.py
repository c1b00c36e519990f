"""AdaptiveMap with its grid resident in GPU memory.

Python face of the reference's ``AdaptiveMap`` (src/vegas/_vegas.pyx:39-832):
same constructor, ``map``/``invmap``/``__call__``/``jac``/``jac1d``,
``add_training_data``, ``adapt``, ``adapt_to_samples``, ``make_uniform``, ``region``,
``extract_grid``, ``settings`` and pickling.  The grid ``[dim, max(ninc)+1]``
and increments live on the device in FP64; every numeric operation is a
kernel of ``libvegas_gb300.so``.  Host (numpy) arguments are copied to the
device and results copied back, so reference-style code keeps working;
CUDA tensors are used in place.
"""
import numpy as np
import torch

from . import _native as N

TINY = 1e-257  # _vegas.pyx:34


def _device(device):
    if device is None:
        if not torch.cuda.is_available():
            raise RuntimeError('vegas_gb300 needs a CUDA device (no CPU fallback)')
        return torch.device('cuda', torch.cuda.current_device())
    return torch.device(device)


class AdaptiveMap(object):
    r"""Adaptive map ``y -> x(y)`` from the unit hypercube, one axis at a time.

    ``grid[d][i]`` are the x-space nodes of direction d; ``ninc`` (number or
    array) regrids to that many increments keeping the map's Jacobian
    (pyx:112-137).
    """

    def __init__(self, grid, ninc=None, device=None):
        if isinstance(grid, AdaptiveMap):
            self.device = grid.device if device is None else _device(device)
            self._ninc = np.array(grid._ninc, np.int64)
            self._grid = grid._grid.to(self.device, copy=True)
            self._inc = grid._inc.to(self.device, copy=True)
        else:
            self.device = _device(device)
            dim = len(grid)
            len_g = np.array([len(x) for x in grid], dtype=np.int64)
            if len(len_g) == 0 or min(len_g) < 2:
                raise ValueError('grid[d] must have at least 2 elements, not {}'.format(
                    min(len_g) if len(len_g) else 0))
            K = int(len_g.max()) - 1
            g = np.zeros((dim, K + 1))
            inc = np.zeros((dim, K))
            for d in range(dim):
                nodes = sorted(float(v) for v in grid[d])
                g[d, :len(nodes)] = nodes
                for i in range(len(nodes) - 1):
                    inc[d, i] = g[d, i + 1] - g[d, i]
            self._ninc = len_g - 1
            self._grid = torch.from_numpy(g).to(self.device)
            self._inc = torch.from_numpy(inc).to(self.device)
        self.sum_f = None
        self.n_f = None
        if ninc is not None and not np.all(np.asarray(ninc) == self._ninc):
            if np.all(self._ninc == 1):
                self.make_uniform(ninc=ninc)
            else:
                self.adapt(ninc=ninc)

    # ---------------------------------------------------------------- info
    @property
    def dim(self):
        return int(self._grid.shape[0])

    @property
    def ninc(self):
        return np.array(self._ninc)

    @property
    def grid(self):
        """Host copy of the grid (rows padded to max(ninc)+1)."""
        return self._grid.cpu().numpy()

    @property
    def inc(self):
        return self._inc.cpu().numpy()

    @property
    def grid_tensor(self):
        """The device grid itself ``[dim, max(ninc)+1]`` (FP64)."""
        return self._grid

    @property
    def inc_tensor(self):
        return self._inc

    def region(self, d=-1):
        g = self.grid
        if d < 0:
            return [self.region(k) for k in range(self.dim)]
        return (g[d, 0], g[d, self._ninc[d]])

    def extract_grid(self):
        g = self.grid
        return [list(g[d, :self._ninc[d] + 1]) for d in range(self.dim)]

    def __reduce__(self):
        return (AdaptiveMap, (self.extract_grid(),))

    def settings(self, ngrid=5):
        g = self.grid
        ans = []
        if ngrid > 0:
            for d in range(self.dim):
                grid_d = np.array(g[d, :self._ninc[d] + 1])
                nskip = int(self._ninc[d] // ngrid)
                if nskip < 1:
                    nskip = 1
                start = nskip // 2
                ans.append('    grid[%2d] = %s' % (d, np.array2string(
                    grid_d[start::nskip], precision=3, prefix='    grid[xx] = ')))
        return '\n'.join(ans) + '\n'

    # --------------------------------------------------------- structure
    def _geom(self):
        return N.i64_array(self._ninc)

    def clear(self):
        """Forget accumulated training data (pyx:596-599)."""
        self.sum_f = None
        self.n_f = None

    def make_uniform(self, ninc=None):
        """Replace the grid by a uniform one with ninc increments (pyx:205-241)."""
        if ninc is None:
            ninc = np.array(self._ninc)
        elif np.shape(ninc) == ():
            ninc = np.full(self.dim, int(ninc), dtype=np.int64)
        elif np.shape(ninc) == (self.dim,):
            ninc = np.asarray(ninc, np.int64)
        else:
            raise ValueError('ninc has wrong shape -- {}'.format(np.shape(ninc)))
        if min(ninc) < 1:
            raise ValueError('no of increments < 1 in AdaptiveMap -- %s' % str(ninc))
        lim = self.region()
        K = int(max(ninc))
        g = torch.zeros((self.dim, K + 1), dtype=torch.float64, device=self.device)
        inc = torch.zeros((self.dim, K), dtype=torch.float64, device=self.device)
        L = N.load()
        N.check(L.vg_make_uniform(self.dim, N.i64_array(ninc), N.dbl_array([a for a, b in lim]),
                                  N.dbl_array([b for a, b in lim]), N.ptr(g), K + 1, N.ptr(inc), K,
                                  N.stream_ptr(self.device)))
        self._grid, self._inc, self._ninc = g, inc, np.array(ninc, np.int64)
        self.clear()

    def adapt(self, alpha=0.0, ninc=None):
        """Adapt the grid to the accumulated training data (pyx:467-594)."""
        dim = self.dim
        if ninc is None:
            new_ninc = np.array(self._ninc)
        elif np.shape(ninc) == ():
            new_ninc = np.full(dim, int(ninc), np.int64)
        elif len(ninc) == dim:
            new_ninc = np.array(ninc, np.int64)
        else:
            raise ValueError('badly formed ninc = ' + str(ninc))
        if min(new_ninc) < 1:
            raise ValueError('ninc < 1: ' + str(list(new_ninc)))
        K = int(max(new_ninc))
        g = torch.zeros((dim, K + 1), dtype=torch.float64, device=self.device)
        inc = torch.zeros((dim, K), dtype=torch.float64, device=self.device)
        L = N.load()
        N.check(L.vg_adapt(dim, N.i64_array(self._ninc), N.i64_array(new_ninc), N.ptr(self._grid),
                           N.ptr(self._inc), self._grid.shape[1], self._inc.shape[1],
                           N.ptr(self.sum_f), N.ptr(self.n_f), float(alpha), N.ptr(g), N.ptr(inc),
                           K + 1, K, N.stream_ptr(self.device)))
        self._grid, self._inc, self._ninc = g, inc, new_ninc
        self.clear()

    # ------------------------------------------------------------- maps
    def _as_device(self, a, dtype=None):
        if isinstance(a, torch.Tensor):
            t = a.to(self.device)
            if dtype is not None:
                t = t.to(dtype)
            return t.contiguous(), True
        arr = np.ascontiguousarray(a, dtype=np.float64 if dtype is None else
                                   {torch.float64: np.float64, torch.float32: np.float32}[dtype])
        return torch.from_numpy(arr).to(self.device), False

    def map(self, y, x, jac, ny=-1):
        """Fill x[j, d] and jac[j] for y[j, d] (pyx:310-360).

        Works in place on CUDA tensors (FP32 or FP64, matching dtypes) or on
        host numpy arrays (computed on the device, copied back)."""
        yt, on_dev = self._as_device(y)
        n = yt.shape[0] if ny < 0 else int(ny)
        if n > yt.shape[0]:
            raise ValueError('ny > y.shape[0]: %d > %d' % (n, yt.shape[0]))
        if yt.dtype not in (torch.float32, torch.float64):
            yt = yt.to(torch.float64)
        dt = N.VG_F64 if yt.dtype == torch.float64 else N.VG_F32
        if on_dev and isinstance(x, torch.Tensor) and isinstance(jac, torch.Tensor):
            xt, jt = x, jac
        else:
            xt = torch.empty_like(yt)
            jt = torch.empty(yt.shape[0], dtype=yt.dtype, device=self.device)
        L = N.load()
        N.check(L.vg_map(self.dim, self._geom(), N.ptr(self._grid), N.ptr(self._inc),
                         self._grid.shape[1], self._inc.shape[1], n, N.ptr(yt), N.ptr(xt),
                         N.ptr(jt), dt, N.stream_ptr(self.device)))
        if xt is not x:
            x[:n] = xt[:n].cpu().numpy() if not isinstance(x, torch.Tensor) else xt[:n]
            jac[:n] = jt[:n].cpu().numpy() if not isinstance(jac, torch.Tensor) else jt[:n]

    def invmap(self, x, y, jac, nx=-1):
        """Fill y[j, d] and jac[j] (= dx/dy) for x[j, d] (pyx:362-413).

        CUDA tensors are used in place; host arrays are computed on the
        device and copied back."""
        xt, on_dev = self._as_device(x)
        n = xt.shape[0] if nx < 0 else int(nx)
        if n > xt.shape[0]:
            raise ValueError('nx > x.shape[0]: %d > %d' % (n, xt.shape[0]))
        if xt.dtype not in (torch.float32, torch.float64):
            xt = xt.to(torch.float64)
        dt = N.VG_F64 if xt.dtype == torch.float64 else N.VG_F32
        if on_dev and isinstance(y, torch.Tensor) and isinstance(jac, torch.Tensor):
            yt, jt = y, jac
        else:
            yt = torch.empty_like(xt)
            jt = torch.empty(xt.shape[0], dtype=xt.dtype, device=self.device)
        L = N.load()
        N.check(L.vg_invmap(self.dim, self._geom(), N.ptr(self._grid), N.ptr(self._inc),
                            self._grid.shape[1], self._inc.shape[1], n, N.ptr(xt), N.ptr(yt),
                            N.ptr(jt), dt, N.stream_ptr(self.device)))
        if yt is not y:
            y[:n] = yt[:n].cpu().numpy() if not isinstance(y, torch.Tensor) else yt[:n]
            jac[:n] = jt[:n].cpu().numpy() if not isinstance(jac, torch.Tensor) else jt[:n]

    def adapt_to_samples(self, x, f, nitn=5, alpha=1.0, nproc=1):
        """Adapt the map to data {x, f(x)} (pyx:728-790): the grid is
        regridded to min(max(ninc, 1000), len(x) / 10) increments, then nitn
        rounds of invmap -> training data (jac f)^2 -> adapt(alpha), and
        finally regridded to max(max(ninc), 1000) increments, as the
        reference does.  ``f`` is a callable (called with ``x`` as given)
        or an array of values; ``nproc`` is accepted for compatibility (the
        device does the work)."""
        xt, _ = self._as_device(x, torch.float64)
        if xt.dim() != 2 or xt.shape[1] != self.dim:
            raise ValueError('incompatible shape of x: {}'.format(tuple(xt.shape)))
        fx = f(x) if callable(f) else f
        ft, _ = self._as_device(fx, torch.float64)
        ft = ft.reshape(-1)
        if ft.shape[0] != xt.shape[0]:
            raise ValueError('shape of x and f(x) mismatch: {} vs {}'.format(
                tuple(xt.shape), tuple(ft.shape)))
        old_ninc = max(int(max(self._ninc)), 1000)   # Integrator.defaults['maxinc_axis']
        tmp_ninc = int(min(old_ninc, xt.shape[0] / 10.))
        if tmp_ninc < 2:
            raise ValueError('not enough samples: {}'.format(xt.shape[0]))
        y = torch.empty_like(xt)
        jac = torch.empty(xt.shape[0], dtype=torch.float64, device=self.device)
        self.adapt(ninc=tmp_ninc)
        for _ in range(int(nitn)):
            self.invmap(xt, y, jac)
            self.add_training_data(y, (jac * ft) ** 2)
            self.adapt(alpha=alpha, ninc=tmp_ninc)
        if tmp_ninc != old_ninc:
            self.adapt(ninc=old_ninc)

    def __call__(self, y):
        """x values for y (any leading shape; last axis is direction)."""
        is_t = isinstance(y, torch.Tensor)
        ya = y if is_t else np.asarray(y, float)
        shape = tuple(ya.shape)
        yt, _ = self._as_device(ya.reshape(-1, shape[-1]))
        xt = torch.empty_like(yt)
        jt = torch.empty(yt.shape[0], dtype=yt.dtype, device=self.device)
        self.map(yt, xt, jt)
        xt = xt.reshape(shape)
        return xt if is_t else xt.cpu().numpy()

    def jac1d(self, y):
        """dx[d]/dy[d] for each direction (pyx:265-295)."""
        is_t = isinstance(y, torch.Tensor)
        ya = y if is_t else np.asarray(y, float)
        shape = tuple(ya.shape)
        yt, _ = self._as_device(ya.reshape(-1, shape[-1]))
        if yt.dtype not in (torch.float32, torch.float64):
            yt = yt.to(torch.float64)
        yt = yt.contiguous()
        out = torch.empty_like(yt)
        L = N.load()
        N.check(L.vg_jac1d(self.dim, self._geom(), N.ptr(self._inc), self._inc.shape[1], yt.shape[0],
                           N.ptr(yt), N.ptr(out), N.VG_F64 if yt.dtype == torch.float64 else N.VG_F32,
                           N.stream_ptr(self.device)))
        out = out.reshape(shape)
        return out if is_t else out.cpu().numpy()

    def jac(self, y):
        j = self.jac1d(y)
        return j.prod(dim=-1) if isinstance(j, torch.Tensor) else np.prod(j, axis=-1)

    def add_training_data(self, y, f, ny=-1):
        """Accumulate training data f at y for the next adapt (pyx:421-464)."""
        yt, _ = self._as_device(y)
        if yt.dtype not in (torch.float32, torch.float64):
            yt = yt.to(torch.float64)
        ft, _ = self._as_device(f, yt.dtype)
        n = yt.shape[0] if ny < 0 else int(ny)
        if n > yt.shape[0]:
            raise ValueError('ny > y.shape[0]: %d > %d' % (n, yt.shape[0]))
        if self.sum_f is None:
            self.sum_f = torch.zeros(self._inc.shape, dtype=torch.float64, device=self.device)
            self.n_f = torch.zeros(self._inc.shape, dtype=torch.int64, device=self.device)
        dt = N.VG_F64 if yt.dtype == torch.float64 else N.VG_F32
        L = N.load()
        N.check(L.vg_add_training_data(self.dim, self._geom(), self._inc.shape[1], n, N.ptr(yt),
                                       N.ptr(ft), dt, N.ptr(self.sum_f), N.ptr(self.n_f),
                                       N.stream_ptr(self.device)))

    def training_data(self):
        """(sum_f, n_f) as host arrays in the reference's convention (n_f + TINY)."""
        if self.sum_f is None:
            return None, None
        return self.sum_f.cpu().numpy(), self.n_f.cpu().numpy().astype(np.float64) + TINY

    def random(self, n=None, generator=None):
        y = torch.rand((1 if n is None else n, self.dim), dtype=torch.float64,
                       device=self.device, generator=generator)
        x = self(y)
        return x[0] if n is None else x
