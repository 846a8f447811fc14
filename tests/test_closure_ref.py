"""The PyTorch restatement of the learned rim (tests/closure_ref.py) against a
direct cell-by-cell evaluation of the closure's formula on a tiny grid, so that
the GPU tests compare the kernels with a reference whose conventions (tap order,
face boxes, depths, gains) are pinned independently of conv3d."""
import numpy as np

import closure_ref as R

PAD = R.PAD


def _direct(fields, zinv, kap, params):
    p = R.bf16(params)
    W1 = p[:R.NW1].reshape(32, 8 * 27)
    W2 = p[R.NW1:R.NW1 + R.NW2].reshape(6, 4, 32, 27)
    G = p[R.NW1 + R.NW2:].reshape(6, 6, 4)
    u, v, w, P = (fields[k].astype(np.float32) for k in range(4))
    pz = P * zinv
    x = R.bf16(np.stack([u, v, w, pz, kap * u, kap * v, kap * w, kap * pz]).astype(np.float32))
    ny, nx, nz = u.shape
    nn = {0: nz, 1: nx, 2: ny}                  # closure axes z, x, y

    def coord(c, A):                             # c = (y, x, z)
        return c[{0: 2, 1: 1, 2: 0}[A]]

    def a_of(f, c):
        A, side = f >> 1, f & 1
        k = coord(c, A)
        return k - (nn[A] - PAD - 1) if side else PAD - k

    def in_box(f, c):
        A = f >> 1
        if not 0 <= a_of(f, c) < 7:
            return False
        return all(4 <= coord(c, B) < nn[B] - 4 for B in range(3) if B != A)

    cache = {}

    def hidden(f, c):
        if not in_box(f, c):
            return np.zeros(32, np.float32)
        key = (f,) + c
        if key not in cache:
            y, xx, z = c
            feats = x[:, y - 1:y + 2, xx - 1:xx + 2, z - 1:z + 2].reshape(8, 27)
            cache[key] = R.bf16(np.maximum(W1 @ feats.reshape(-1), 0.0))
        return cache[key]

    out = np.zeros((4, ny, nx, nz), np.float64)
    mask = R.rim_mask((ny, nx, nz))
    for c in zip(*np.nonzero(mask)):
        c = tuple(int(i) for i in c)
        for A in range(3):
            k = coord(c, A)
            if 4 <= k < PAD:
                f = 2 * A
            elif nn[A] - PAD <= k < nn[A] - 4:
                f = 2 * A + 1
            else:
                continue
            depth = a_of(f, c) - 1
            yv = np.zeros(4)
            for t in range(27):
                dy, dx, dz = t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1
                yv += W2[f][:, :, t] @ hidden(f, (c[0] + dy, c[1] + dx, c[2] + dz))
            out[:, c[0], c[1], c[2]] += G[f][depth] * yv
    out[3] /= np.where(zinv > 0, zinv, 1.0)
    return out


def test_torch_restatement_matches_the_direct_formula():
    rng = np.random.default_rng(7)
    shape = (2 * PAD + 2, 2 * PAD + 1, 2 * PAD + 3)   # a 1x2x3 (x, y, z... as y, x, z) model
    fields = np.zeros((4,) + shape, np.float32)
    inner = (slice(4, -4),) * 3
    for k in range(4):
        fields[k][inner] = rng.standard_normal(fields[k][inner].shape)
    vel = rng.uniform(1500, 4500, shape).astype(np.float32)
    rho = rng.uniform(1800, 2500, shape).astype(np.float32)
    fields[3] *= 1e6
    zinv, kap = R.scales(vel, rho, np.float32(0.4 / 4500.0))
    params = rng.standard_normal(R.NW1 + R.NW2 + R.NG).astype(np.float32) * 0.2
    ref = R.closure(fields, zinv, kap, params)
    direct = _direct(fields, zinv, kap, params)
    mask = R.rim_mask(shape)
    assert not np.any(ref[:, ~mask])
    for k in range(4):
        scale = np.abs(direct[k]).max()
        assert scale > 0
        assert np.abs(ref[k] - direct[k]).max() <= 1e-3 * scale, k


def test_rim_and_face_box_counts():
    shape = (30, 27, 33)                          # (y, x, z)
    nn = np.array([33, 27, 30])                   # (z, x, y)
    rim = R.rim_mask(shape).sum()
    assert rim == np.prod(nn - 8) - np.prod(nn - 20)
    for f in range(6):
        ax, sl, rimsl, depth = R._face_slices(shape, f)
        ext = [s.stop - s.start for s in sl]
        assert ext[ax] == 7 and rimsl.stop - rimsl.start == 6 and sorted(depth) == list(range(6))
