"""Learned proposal: a coupling-layer normalising flow composed after the
AdaptiveMap (no counterpart in the reference).

``Flow`` owns the parameters (FP32 master copy + BF16 tensor-core mirrors) in
device memory; every computation is a kernel of libvegas_gb300.so:
``sample`` (zhat -> z, sampling direction), ``density`` (z -> zhat,
log q), ``train_step`` (forward + backward + Adam on the variance loss
-sum_i w_i log q(z_i) with w_i = (f_i J_i)^2 from vegas's own samples).
"""
import ctypes
import math

import numpy as np
import torch

from . import _native as N


class Flow(object):
    """Piecewise-quadratic coupling flow on the unit cube.

    Args:
        dim: dimension (<= 16).
        nlayers: coupling layers (<= 8), K: spline bins (<= 64), hidden: 128.
        seed: initialisation seed.  W3 starts at zero, so the initial flow is
            the identity map.
    """

    def __init__(self, dim, nlayers=6, K=32, hidden=128, seed=0, device=None, lr=1e-3):
        if device is None:
            device = torch.device('cuda', torch.cuda.current_device())
        self.device = torch.device(device)
        self.dim, self.nlayers, self.K, self.hidden = int(dim), int(nlayers), int(K), int(hidden)
        L = N.load()
        self.nparams = int(L.vg_flow_nparams(self.dim, self.nlayers, self.K, self.hidden))
        if self.nparams < 0:
            N.check(N.VG_ERR_UNSUPPORTED)
        nm = int(L.vg_flow_mirror_elems(self.dim, self.nlayers, self.K, self.hidden))
        theta = _init_theta(self.dim, self.nlayers, self.K, self.hidden, seed)
        dev = self.device
        self.theta = torch.from_numpy(theta).to(dev)
        self.mirror = torch.zeros(nm, dtype=torch.int16, device=dev)
        self.grad = torch.zeros(self.nparams, dtype=torch.float32, device=dev)
        self.adam_m = torch.zeros(self.nparams, dtype=torch.float32, device=dev)
        self.adam_v = torch.zeros(self.nparams, dtype=torch.float32, device=dev)
        self.loss = torch.zeros(1, dtype=torch.float64, device=dev)
        self.step_count = 0
        self.lr = lr
        self._work = None
        self.refresh()

    def _struct(self):
        s = N.VgFlow()
        s.dim, s.nlayers, s.K, s.hidden = self.dim, self.nlayers, self.K, self.hidden
        s.theta = self.theta.data_ptr()
        s.mirror = self.mirror.data_ptr()
        s.grad = self.grad.data_ptr()
        s.adam_m = self.adam_m.data_ptr()
        s.adam_v = self.adam_v.data_ptr()
        s.loss = self.loss.data_ptr()
        return s

    def refresh(self):
        """Rebuild the BF16 mirrors after theta changed."""
        N.check(N.load().vg_flow_refresh(ctypes.byref(self._struct()), N.stream_ptr(self.device)))

    def set_theta(self, theta):
        self.theta.copy_(torch.as_tensor(np.asarray(theta, np.float32)))
        self.refresh()

    def sample(self, zhat, z=None, ld=None):
        """zhat [n, dim] (float32, unit cube) -> (z, logdet), log|dz/dzhat| = -logdet.
        z, ld: optional output tensors ([n, dim] and [n] float32)."""
        zhat = zhat.to(self.device, torch.float32).contiguous()
        n = zhat.shape[0]
        if z is None:
            z = torch.empty_like(zhat)
        if ld is None:
            ld = torch.empty(n, dtype=torch.float32, device=self.device)
        N.check(N.load().vg_flow_sample(ctypes.byref(self._struct()), n, N.ptr(zhat), N.ptr(z),
                                        N.ptr(ld), N.stream_ptr(self.device)))
        return z, ld

    def density(self, z):
        """z [n, dim] -> (zhat, logdet = log q_flow(z))."""
        z = z.to(self.device, torch.float32).contiguous()
        n = z.shape[0]
        zh = torch.empty_like(z)
        ld = torch.empty(n, dtype=torch.float32, device=self.device)
        N.check(N.load().vg_flow_density(ctypes.byref(self._struct()), n, N.ptr(z), N.ptr(zh),
                                         N.ptr(ld), N.stream_ptr(self.device)))
        return zh, ld

    def accumulate_grad(self, z, w):
        """grad += d/dtheta [-sum_i w_i log q(z_i)]; loss += the same sum."""
        z = z.to(self.device, torch.float32).contiguous()
        w = w.to(self.device, torch.float32).contiguous()
        n = z.shape[0]
        L = N.load()
        st = self._struct()
        need = int(L.vg_flow_train_bytes(ctypes.byref(st), n))
        if self._work is None or self._work.numel() < need:
            self._work = torch.empty(need, dtype=torch.uint8, device=self.device)
        N.check(L.vg_flow_grad(ctypes.byref(st), n, N.ptr(z), N.ptr(w), N.ptr(self._work),
                               self._work.numel(), N.stream_ptr(self.device)))

    def train_step_normalized(self, z, w, lr=None, clip=10.0):
        """One Adam step on -sum_i w_i log q(z_i) / m with weights already
        normalised to mean 1 (vg_flow_train_batch); only library kernels run."""
        m = z.shape[0]
        N.check(N.load().vg_flow_zero_grad(ctypes.byref(self._struct()), N.stream_ptr(self.device)))
        self.accumulate_grad(z, w)
        self.step_count += 1
        N.check(N.load().vg_flow_adam(ctypes.byref(self._struct()), 1.0 / m,
                                      self.lr if lr is None else lr, 0.9, 0.999, 1e-8,
                                      self.step_count, clip, N.stream_ptr(self.device)))

    def train_step(self, z, w, lr=None, clip=10.0):
        """One Adam step on the loss -sum_i w_i log q(z_i) / sum_i w_i.

        w is rescaled to mean 1 before it reaches the kernels (the BF16
        gradient tensors keep FP32's exponent range, but sums of raw
        (f J)^2 can be huge).  Returns the loss of the batch before the step.
        """
        w = w.to(self.device, torch.float32)
        n = w.shape[0]
        wm = w.mean()
        w = w / torch.clamp(wm, min=1e-30)
        self.grad.zero_()
        self.loss.zero_()
        self.accumulate_grad(z, w)
        self.step_count += 1
        N.check(N.load().vg_flow_adam(ctypes.byref(self._struct()), 1.0 / n,
                                      self.lr if lr is None else lr, 0.9, 0.999, 1e-8,
                                      self.step_count, clip, N.stream_ptr(self.device)))
        return self.loss / n


def _init_theta(dim, nlayers, K, hidden, seed):
    """He-scaled W1, W2; zero W3 and biases (identity flow at start)."""
    rng = np.random.default_rng(seed)
    # layer sizes as in the library (masks by bit pattern)
    nbits = max(1, int(math.ceil(math.log2(dim)))) if dim > 1 else 1
    out = []
    for l in range(nlayers):
        b = (l // 2) % nbits
        B = [i for i in range(dim) if ((i >> b) & 1) == (l % 2)]
        A = [i for i in range(dim) if i not in B]
        if not A or not B:
            A, B = [], list(range(dim))
        dA = max(len(A), 1)
        P = len(B) * (2 * K + 1)
        out.append(rng.normal(0, math.sqrt(2.0 / dA), hidden * dA))
        out.append(np.zeros(hidden))
        out.append(rng.normal(0, math.sqrt(2.0 / hidden), hidden * hidden))
        out.append(np.zeros(hidden))
        out.append(np.zeros(P * hidden))
        out.append(np.zeros(P))
    return np.concatenate(out).astype(np.float32)
