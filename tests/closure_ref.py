"""Plain PyTorch float32 restatement of the learned rim (test infrastructure).

The closure of csrc/a3d_closure.h written with torch.nn.functional.conv3d on one
face box at a time: relu(W1 * x) on the box (inputs cropped one cell wider), the
hidden box zero-padded by one cell, W2_f * h, the per-depth gains on the rim
cells, summed over faces.  Weights and hidden activations are rounded to
bfloat16 as the kernels do (straight through for autograd), inputs too, so the reference
differs from the kernels only in float summation order.  Arrays are
[channel, y, x, z] on the dense rim grid (model + 10 cells per face).
"""
import numpy as np
import torch
import torch.nn.functional as F

PAD, RIM = 10, 6
NW1, NW2, NG = 32 * 8 * 27, 6 * 4 * 32 * 27, 6 * 6 * 4
AX = {0: 2, 1: 1, 2: 0}  # closure axis (z, x, y) -> array axis of [y, x, z]


def bf16(a):
    """Round float32 values to the nearest bfloat16 (ties to even), as float32."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return u.view(np.float32)


def _bf16_t(t):
    return t + (torch.from_numpy(bf16(t.detach().numpy())) - t).detach()


def scales(vel_pad, rho_pad, courant):
    """zinv = 1/(rho vp), kappa = vp * courant on the padded grid (float32 arithmetic)."""
    z = (rho_pad * vel_pad).astype(np.float32)
    zinv = np.where(z > 0, np.float32(1.0) / z, np.float32(0.0)).astype(np.float32)
    return zinv, (vel_pad * np.float32(courant)).astype(np.float32)


def pad_model(m, pad=PAD):
    """Edge replication of a (y, x, z) model by pad cells per face."""
    return np.pad(m, pad, mode="edge").astype(np.float32)


def rim_mask(shape):
    m = np.zeros(shape, bool)
    m[4:-4, 4:-4, 4:-4] = True
    m[PAD:-PAD, PAD:-PAD, PAD:-PAD] = False
    return m


def _face_slices(shape, f):
    """Array slices of face f's box and the box-local rim slice and depths."""
    A, side = f >> 1, f & 1
    ax = AX[A]
    nn = shape[ax]
    sl = [slice(4, s - 4) for s in shape]
    if side == 0:
        sl[ax] = slice(4, PAD + 1)                       # cells 4..10: depth 5..-1
        rim = slice(0, RIM)                              # local 0..5 -> depth 5..0
        depth = np.arange(RIM)[::-1].copy()
    else:
        sl[ax] = slice(nn - PAD - 1, nn - 4)             # depth -1..5
        rim = slice(1, RIM + 1)
        depth = np.arange(RIM)
    return ax, sl, rim, depth


def closure(fields, zinv, kap, params, grad=False):
    """Correction [4, y, x, z] (channel 3 in pressure units) of the closure; with
    grad=True returns (correction in balanced units, params tensor) for autograd."""
    p = torch.tensor(bf16(params), requires_grad=grad)
    W1 = p[:NW1].reshape(32, 8, 3, 3, 3)
    W2 = p[NW1:NW1 + NW2].reshape(6, 4, 32, 3, 3, 3)
    G = p[NW1 + NW2:].reshape(6, 6, 4)
    f32 = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32))
    u, v, w, P = (f32(fields[k]) for k in range(4))
    zi, ka = f32(zinv), f32(kap)
    pz = P * zi
    x = torch.stack([u, v, w, pz, ka * u, ka * v, ka * w, ka * pz])
    x = torch.from_numpy(bf16(x.numpy()))  # bfloat16 inputs
    shape = tuple(u.shape)
    out = torch.zeros((4,) + shape)
    for f in range(6):
        ax, sl, rim, depth = _face_slices(shape, f)
        wide = [slice(s.start - 1, s.stop + 1) for s in sl]
        xb = x[(slice(None),) + tuple(wide)]
        h = F.relu(F.conv3d(xb[None], W1))[0]
        h = _bf16_t(h) if grad else torch.from_numpy(bf16(h.detach().numpy()))
        y = F.conv3d(F.pad(h[None], (1, 1, 1, 1, 1, 1)), W2[f])[0]          # [4, box]
        idx = [slice(None)] * 4
        idx[ax + 1] = rim
        yr = y[tuple(idx)]
        gshape = [1, 1, 1, 1]
        gshape[ax + 1] = RIM
        gains = G[f][torch.from_numpy(depth)].T.reshape([4] + gshape[1:])  # [4, ...] along ax
        osl = list(sl)
        s0 = sl[ax].start
        osl[ax] = slice(s0 + rim.start, s0 + rim.stop)
        out[(slice(None),) + tuple(osl)] = out[(slice(None),) + tuple(osl)] + gains * yr
    if grad:
        return out, p
    res = out.detach().numpy().copy()
    res[3] = res[3] / zinv
    res[3][~np.isfinite(res[3])] = 0.0
    return res


def loss_and_grad(X, T, zinv, kap, params):
    """Loss of one sample and its gradient with respect to the parameters."""
    mask = torch.from_numpy(rim_mask(X.shape[1:]))
    d, p = closure(X, zinv, kap, params, grad=True)
    zi = torch.from_numpy(zinv)
    Xt, Tt = torch.from_numpy(X), torch.from_numpy(T)
    tg = Tt - Xt
    tg = torch.cat([tg[:3], (tg[3] * zi)[None]])
    xb = torch.cat([Xt[:3], (Xt[3] * zi)[None]])
    E = (xb ** 2 * mask).sum()
    L = ((d - tg) ** 2 * mask).sum() / E
    L.backward()
    return float(L), p.grad.numpy().copy()


def std_step(S0, rho_pad, vel_pad, dtx, dty, dtz):
    """The engine's undamped step on the rim grid in float64 (u, v, w then P)."""
    k = np.array([1.196289, -0.0797526, 0.009570313, -0.0006975447], np.float64)
    u0, v0, w0, P0 = (S0[i].astype(np.float64) for i in range(4))
    rho, vp = rho_pad.astype(np.float64), vel_pad.astype(np.float64)
    sh = S0.shape[1:]
    inner = tuple(slice(4, s - 4) for s in sh)

    def dplus(a, ax):
        r = np.zeros(sh)
        for m in range(4):
            r += k[m] * (np.roll(a, -(m + 1), ax) - np.roll(a, m, ax))
        return r

    def dminus(a, ax):
        r = np.zeros(sh)
        for m in range(4):
            r += k[m] * (np.roll(a, -m, ax) - np.roll(a, m + 1, ax))
        return r

    X = np.zeros((4,) + sh)
    ri = 1.0 / rho
    X[0][inner] = (u0 - dtx * dplus(P0, 1) * ri)[inner]
    X[1][inner] = (v0 - dty * dplus(P0, 0) * ri)[inner]
    X[2][inner] = (w0 - dtz * dplus(P0, 2) * ri)[inner]
    t = rho * vp * vp
    X[3][inner] = (P0 - t * (dtx * dminus(X[0], 1) + dty * dminus(X[1], 0) + dtz * dminus(X[2], 2)))[inner]
    return X
