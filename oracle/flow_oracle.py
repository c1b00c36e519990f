"""FP64 restatement of the coupling-layer flow (TEST INFRASTRUCTURE ONLY).

The reference has no learned proposal; this module is the oracle the GPU
flow kernels (vegas_gb300/csrc/vg_flow.cu) are checked against: the same
parameter layout, masks, piecewise-quadratic spline (Mueller et al., "Neural
Importance Sampling", ACM TOG 2019, section 4: bin widths from a softmax,
vertex heights exp()-ed and normalised so the piecewise-linear density
integrates to one), the same log-determinants and the same training loss,
in torch float64 with autograd for the gradients.

Conventions (shared with the kernels):
* density direction (training): x (sample, unit cube) -> layer 0 CDF -> ...
  -> layer L-1 CDF -> xhat; logdet = sum of log PDF of every transformed
  coordinate; log q_flow(x) = logdet.
* sampling direction: xhat -> inverse CDF of layer L-1 -> ... -> layer 0 ->
  x, with log |dx/dxhat| = -logdet(x).
* conditioner of layer l: out = W3 relu(W2 relu(W1 x_A + b1) + b2) + b3,
  out[j*(2K+1) + k] (k < K) width logits of transformed dim j,
  out[j*(2K+1) + K + k] (k <= K) vertex logits.
* loss(theta) = - sum_i w_i logdet_theta(x_i) / sum_i w_i with fixed weights
  w_i = (f_i J_i)^2: its gradient is the variance gradient of the importance
  sampling estimator (up to a positive factor).
"""
import math

import numpy as np
import torch

EPS_W = 1e-3   # minimum bin width fraction: W = EPS_W + (1 - K*EPS_W) softmax


def init_theta(dim, nlayers=6, K=32, hidden=128, seed=0, scale=1.0, out_scale=0.0):
    """Initial parameters: He-scaled W1, W2; W3 = out_scale * N(0, 1/hidden) (0 gives the
    identity transform: equal bin widths and heights)."""
    rng = np.random.default_rng(seed)
    theta = np.zeros(nparams(dim, nlayers, K, hidden), np.float32)
    o = 0
    for s in layer_sizes(dim, nlayers, K, hidden):
        for name, fan in (('W1', s['dA']), ('b1', 0), ('W2', hidden), ('b2', 0),
                          ('W3', hidden), ('b3', 0)):
            n = s[name]
            if name == 'W3':
                theta[o:o + n] = out_scale * rng.normal(0, 1 / math.sqrt(fan), n)
            elif fan:
                theta[o:o + n] = scale * rng.normal(0, math.sqrt(2.0 / fan), n)
            o += n
    return theta


def masks(dim, nlayers):
    """(A, B) index lists per layer: bit b = (l//2) % nbits of the index,
    B = indices whose bit equals l % 2."""
    nbits = max(1, int(math.ceil(math.log2(dim))))
    out = []
    for l in range(nlayers):
        b = (l // 2) % nbits
        B = [i for i in range(dim) if ((i >> b) & 1) == (l % 2)]
        A = [i for i in range(dim) if i not in B]
        if not A or not B:   # degenerate (dim 1): condition on nothing
            A, B = [], list(range(dim))
        out.append((A, B))
    return out


def layer_sizes(dim, nlayers, K, hidden):
    sizes = []
    for A, B in masks(dim, nlayers):
        dA, dB = max(len(A), 1), len(B)
        P = dB * (2 * K + 1)
        sizes.append(dict(dA=dA, dB=dB, P=P, W1=hidden * dA, b1=hidden, W2=hidden * hidden,
                          b2=hidden, W3=P * hidden, b3=P))
    return sizes


def nparams(dim, nlayers=6, K=32, hidden=128):
    return sum(s['W1'] + s['b1'] + s['W2'] + s['b2'] + s['W3'] + s['b3']
               for s in layer_sizes(dim, nlayers, K, hidden))


def unpack(theta, dim, nlayers=6, K=32, hidden=128):
    """Flat parameter vector -> per-layer dict of tensors (views)."""
    layers, o = [], 0
    for s in layer_sizes(dim, nlayers, K, hidden):
        L = {}
        for name, shape in (('W1', (hidden, s['dA'])), ('b1', (hidden,)),
                            ('W2', (hidden, hidden)), ('b2', (hidden,)),
                            ('W3', (s['P'], hidden)), ('b3', (s['P'],))):
            n = int(np.prod(shape))
            L[name] = theta[o:o + n].reshape(shape)
            o += n
        layers.append(L)
    return layers


def spline_tables(wlog, vlog, K):
    """Widths W[.., K], normalised vertex heights V[.., K+1], bin edges E,
    cumulative CDF at the edges Cb."""
    s = torch.softmax(wlog, dim=-1)
    W = EPS_W + (1 - K * EPS_W) * s
    u = torch.exp(vlog)
    seg = 0.5 * (u[..., :-1] + u[..., 1:]) * W
    Z = seg.sum(dim=-1, keepdim=True)
    V = u / Z
    E = torch.cat([torch.zeros_like(W[..., :1]), torch.cumsum(W, dim=-1)], dim=-1)
    Cb = torch.cat([torch.zeros_like(W[..., :1]), torch.cumsum(seg / Z, dim=-1)], dim=-1)
    return W, V, E, Cb


def spline_cdf(x, wlog, vlog, K):
    W, V, E, Cb = spline_tables(wlog, vlog, K)
    b = torch.clamp(torch.searchsorted(E[..., 1:-1].contiguous(), x.unsqueeze(-1),
                                       right=True).squeeze(-1), 0, K - 1)
    g = lambda t, idx: torch.gather(t, -1, idx.unsqueeze(-1)).squeeze(-1)  # noqa: E731
    Wb, Eb, Vb, Vb1, Cbb = g(W, b), g(E, b), g(V, b), g(V, b + 1), g(Cb, b)
    a = (x - Eb) / Wb
    C = Cbb + Wb * (a * Vb + 0.5 * a * a * (Vb1 - Vb))
    pdf = Vb + a * (Vb1 - Vb)
    return C, torch.log(pdf)


def spline_inverse(c, wlog, vlog, K):
    W, V, E, Cb = spline_tables(wlog, vlog, K)
    b = torch.clamp(torch.searchsorted(Cb[..., 1:-1].contiguous(), c.unsqueeze(-1),
                                       right=True).squeeze(-1), 0, K - 1)
    g = lambda t, idx: torch.gather(t, -1, idx.unsqueeze(-1)).squeeze(-1)  # noqa: E731
    Wb, Eb, Vb, Vb1, Cbb = g(W, b), g(E, b), g(V, b), g(V, b + 1), g(Cb, b)
    qa = 0.5 * Wb * (Vb1 - Vb)
    qb = Wb * Vb
    r = c - Cbb
    a = 2 * r / (qb + torch.sqrt(torch.clamp(qb * qb + 4 * qa * r, min=0.0)))
    x = Eb + a * Wb
    pdf = Vb + a * (Vb1 - Vb)
    return x, torch.log(pdf)


BF16 = False   # emulate the GPU's BF16 operands of the two MMA layers


def _bf16(t):
    return t.to(torch.bfloat16).to(t.dtype) if BF16 else t


def conditioner(L, xA):
    h1 = _bf16(torch.relu(xA @ L['W1'].T + L['b1']))
    h2 = _bf16(torch.relu(h1 @ _bf16(L['W2']).T + L['b2']))
    return h2 @ _bf16(L['W3']).T + L['b3']


def density_pass(theta, x, dim, nlayers=6, K=32, hidden=128):
    """x [n, dim] -> (xhat, logdet)."""
    layers = unpack(theta, dim, nlayers, K, hidden)
    z = x.clone()
    logdet = torch.zeros(x.shape[0], dtype=x.dtype)
    for L, (A, B) in zip(layers, masks(dim, nlayers)):
        xA = z[:, A] if A else torch.zeros((z.shape[0], 1), dtype=z.dtype)
        out = conditioner(L, xA).reshape(z.shape[0], len(B), 2 * K + 1)
        C, lp = spline_cdf(z[:, B], out[..., :K], out[..., K:], K)
        z = z.clone()
        z[:, B] = C
        logdet = logdet + lp.sum(dim=1)
    return z, logdet


def sample_pass(theta, xhat, dim, nlayers=6, K=32, hidden=128):
    """xhat [n, dim] -> (x, logdet(x)); log |dx/dxhat| = -logdet."""
    layers = unpack(theta, dim, nlayers, K, hidden)
    z = xhat.clone()
    logdet = torch.zeros(xhat.shape[0], dtype=xhat.dtype)
    ms = masks(dim, nlayers)
    for l in reversed(range(nlayers)):
        L, (A, B) = layers[l], ms[l]
        xA = z[:, A] if A else torch.zeros((z.shape[0], 1), dtype=z.dtype)
        out = conditioner(L, xA).reshape(z.shape[0], len(B), 2 * K + 1)
        xb, lp = spline_inverse(z[:, B], out[..., :K], out[..., K:], K)
        z = z.clone()
        z[:, B] = xb
        logdet = logdet + lp.sum(dim=1)
    return z, logdet


def loss_and_grad(theta_np, x_np, w_np, dim, nlayers=6, K=32, hidden=128):
    """Loss -sum w logdet / sum w and its gradient (float64 autograd)."""
    theta = torch.tensor(np.asarray(theta_np, np.float64), requires_grad=True)
    x = torch.tensor(np.asarray(x_np, np.float64))
    w = torch.tensor(np.asarray(w_np, np.float64))
    _, ld = density_pass(theta, x, dim, nlayers, K, hidden)
    loss = -(w * ld).sum() / w.sum()
    loss.backward()
    return float(loss), theta.grad.numpy()
