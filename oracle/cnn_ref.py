"""CPU oracle of the learned preconditioner network and the flexible PCG solver.

Test infrastructure only: the product path is the CUDA implementation in
csrc/cnn.cu and csrc/lpcg.cu; nothing here is imported by the library.

The reference has no learned component: this oracle defines the network the
library implements, in FP64, so the GPU forward pass, its gradients and one
optimiser step can be checked against an independent implementation, and so
the solver can be checked against a plain restatement of flexible CG.

Network (complex image in, complex image out, 2 real channels):
  s  = sqrt(mean |r|^2)                 (per image; s = 0 gives z = 0)
  a0 = [re(r), im(r)] / s
  a_{l+1} = relu(conv3x3(a_l, W_l))     l = 0..4, channels 2->32->32->32->32->32
                                        (identity instead of relu when linear=True)
  v  = conv3x3(a_5, W_5) + skip * a0    32 -> 2
  z  = s * (v[0] + i v[1])
conv3x3: zero padding, stride 1, no bias, cross-correlation
  out[co, y, x] = sum_ci sum_ky sum_kx W[co, ci, ky, kx] in[ci, y+ky-1, x+kx-1]
where x is the first (fastest, MATLAB row) image index and y the second.
Parameter vector: W_0 .. W_5 flattened in [co][ci][ky][kx] order, then skip.
"""
from __future__ import annotations

import numpy as np

CHANNELS = (2, 32, 32, 32, 32, 32, 2)


def n_params(channels=CHANNELS):
    return sum(channels[l + 1] * channels[l] * 9 for l in range(len(channels) - 1)) + 1


def unpack(theta, channels=CHANNELS):
    Ws, o = [], 0
    for l in range(len(channels) - 1):
        n = channels[l + 1] * channels[l] * 9
        Ws.append(np.asarray(theta[o:o + n], dtype=np.float64).reshape(channels[l + 1], channels[l], 3, 3))
        o += n
    return Ws, float(theta[o])


def init_params(seed, channels=CHANNELS):
    """He-normal initial weights (std sqrt(2 / (9 cin))), skip = 0; numpy PCG64(seed)."""
    g = np.random.Generator(np.random.PCG64(seed))
    parts = []
    for l in range(len(channels) - 1):
        cin, cout = channels[l], channels[l + 1]
        parts.append(g.standard_normal(cout * cin * 9) * np.sqrt(2.0 / (9 * cin)))
    parts.append(np.zeros(1))
    return np.concatenate(parts).astype(np.float32)


def conv3x3(a, W):
    """a [B, cin, Y, X], W [cout, cin, 3, 3] -> [B, cout, Y, X] (zero padding)."""
    B, cin, Y, X = a.shape
    p = np.zeros((B, cin, Y + 2, X + 2), dtype=np.float64)
    p[:, :, 1:-1, 1:-1] = a
    out = np.zeros((B, W.shape[0], Y, X), dtype=np.float64)
    for ky in range(3):
        for kx in range(3):
            out += np.einsum("oc,bcyx->boyx", W[:, :, ky, kx], p[:, :, ky:ky + Y, kx:kx + X])
    return out


def conv3x3_wgrad(a, g):
    """dW[co, ci, ky, kx] = sum_b,y,x g[b, co, y, x] a[b, ci, y+ky-1, x+kx-1]."""
    B, cin, Y, X = a.shape
    p = np.zeros((B, cin, Y + 2, X + 2), dtype=np.float64)
    p[:, :, 1:-1, 1:-1] = a
    dW = np.zeros((g.shape[1], cin, 3, 3), dtype=np.float64)
    for ky in range(3):
        for kx in range(3):
            dW[:, :, ky, kx] = np.einsum("boyx,bcyx->oc", g, p[:, :, ky:ky + Y, kx:kx + X])
    return dW


def conv3x3_dgrad(g, W):
    """Gradient w.r.t. the conv input: correlation of g with the flipped, transposed kernel."""
    Wt = W[:, :, ::-1, ::-1].transpose(1, 0, 2, 3)
    return conv3x3(g, Wt)


def _planes(r):
    """Complex images [B, X, Y] (x fastest in memory order F) -> [B, 2, Y, X] and scales s [B]."""
    r = np.asarray(r, dtype=np.complex128)
    s = np.sqrt(np.mean(np.abs(r) ** 2, axis=(1, 2)))
    inv = np.where(s > 0, 1.0 / np.where(s > 0, s, 1.0), 0.0)
    a0 = np.stack([r.real, r.imag], axis=1).transpose(0, 1, 3, 2) * inv[:, None, None, None]
    return a0, s


def forward(theta, r, channels=CHANNELS, keep=False, linear=False):
    """z = net(r) for r [B, X, Y] complex; returns z [B, X, Y] (and the activations if keep)."""
    Ws, skip = unpack(theta, channels)
    a0, s = _planes(r)
    acts = [a0]
    a = a0
    for l, W in enumerate(Ws):
        pre = conv3x3(a, W)
        a = np.maximum(pre, 0.0) if (l < len(Ws) - 1 and not linear) else pre
        acts.append(a)
    v = a + skip * a0
    zt = v.transpose(0, 1, 3, 2)
    z = (zt[:, 0] + 1j * zt[:, 1]) * s[:, None, None]
    if keep:
        return z, acts, s
    return z


def forward_extended(theta, r, channels=CHANNELS, linear=True):
    """The network on the zero-extended image: r padded by L zeros on each side (L = layers, the
    receptive-field radius), the network applied, the centre cropped.  Intermediate activations
    outside the image are then whatever the layers compute there (not forced to zero), which is the
    operator that crops reaching past the image edge train, and, for a linear network, the single
    folded (2L+1)^2 filter."""
    L = len(channels) - 1
    r = np.asarray(r)
    B, X, Y = r.shape
    rp = np.zeros((B, X + 2 * L, Y + 2 * L), dtype=np.complex128)
    rp[:, L:L + X, L:L + Y] = r
    # the network is positively homogeneous, so the input normalisation does not change z
    return forward(theta, rp, channels, linear=linear)[:, L:L + X, L:L + Y]


def loss_and_grad(theta, r, e, margin, channels=CHANNELS, kind="rel", linear=False):
    """Loss over the interior mask m (margin pixels dropped on every side) and dL/dtheta.

    kind "rel": L = mean_b ||m (z_b - e_b)||^2 / ||m e_b||^2
    kind "cos": L = mean_b 1 - |<m z_b, m e_b>|^2 / (||m z_b||^2 ||m e_b||^2), invariant to a complex
                scale of z_b (flexible CG's line search fixes the scale of each direction).
    """
    Ws, skip = unpack(theta, channels)
    z, acts, s = forward(theta, r, channels, keep=True, linear=linear)
    B, X, Y = z.shape
    m = np.zeros((X, Y))
    m[margin:X - margin, margin:Y - margin] = 1.0
    e = np.asarray(e, dtype=np.complex128)
    den = np.sum(m * np.abs(e) ** 2, axis=(1, 2))
    den = np.where(den > 0, den, 1.0)
    if kind == "rel":
        diff = m * (z - e)
        L = float(np.mean(np.sum(np.abs(diff) ** 2, axis=(1, 2)) / den))
        gz = 2.0 * diff / den[:, None, None] / B                     # dL/d(re z) + i dL/d(im z)
    else:
        zm, em = m * z, m * e
        Z = np.sum(np.abs(zm) ** 2, axis=(1, 2))
        c = np.sum(np.conj(zm) * em, axis=(1, 2))
        ok = Z > 0
        Zs = np.where(ok, Z, 1.0)
        L = float(np.mean(np.where(ok, 1.0 - np.abs(c) ** 2 / (Zs * den), 1.0)))
        gz = (-2.0 * np.conj(c)[:, None, None] * em / (Zs * den)[:, None, None]
              + 2.0 * (np.abs(c) ** 2)[:, None, None] * zm / (Zs ** 2 * den)[:, None, None]) / B
        gz = np.where(ok[:, None, None], gz, 0.0)
    gv = np.stack([gz.real, gz.imag], axis=1).transpose(0, 1, 3, 2) * s[:, None, None, None]
    grads = [None] * len(Ws)
    dskip = float(np.sum(gv * acts[0]))
    g = gv
    for l in range(len(Ws) - 1, -1, -1):
        grads[l] = conv3x3_wgrad(acts[l], g)
        if l > 0:
            g = conv3x3_dgrad(g, Ws[l])
            if not linear:
                g = g * (acts[l] > 0)
    flat = np.concatenate([gw.reshape(-1) for gw in grads] + [np.array([dskip])])
    return L, flat


def adam_step(theta, grad, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (t counts from 1); returns new (theta, m, v)."""
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    return theta - lr * mh / (np.sqrt(vh) + eps), m, v


def fcg_ref(normal, b, precond, nit, lam=0.0, x0=None, gtruth=None, m=1):
    """Flexible PCG (FCG(m)) on (H + lam I) x = b with H = normal(.) Hermitian and z = precond(r).

      alpha = (p' r) / (p' q),  q = (H + lam) p      exact line search along p
      p_new = z - sum_j (q_j' z) / (p_j' q_j) p_j    z conjugated against the last m directions
    With precond = identity this is CG.  Returns (x, res_sq history, nrmse history).
    """
    b = np.asarray(b, dtype=np.complex128)
    x = np.zeros_like(b) if x0 is None else np.asarray(x0, dtype=np.complex128).copy()
    Hx = lambda v: normal(v) + lam * v
    r = b - Hx(x)
    z = precond(r)
    p = z.copy()
    res, err = [float(np.vdot(r, r).real)], []
    gn = None if gtruth is None else np.linalg.norm(gtruth)
    if gtruth is not None:
        err.append(float(np.linalg.norm(x - gtruth) / gn))
    hist = []
    for _ in range(nit):
        q = Hx(p)
        pq = np.vdot(p, q)
        alpha = np.vdot(p, r) / pq
        x = x + alpha * p
        r = r - alpha * q
        hist = (hist + [(p, q, pq)])[-m:]
        z = precond(r)
        p = z.copy()
        for pj, qj, pqj in hist:
            p = p - (np.vdot(qj, z) / pqj) * pj
        res.append(float(np.vdot(r, r).real))
        if gtruth is not None:
            err.append(float(np.linalg.norm(x - gtruth) / gn))
    return x, np.array(res), np.array(err)
