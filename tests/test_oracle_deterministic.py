"""The oracle's deterministic grid mass (svo_deterministic_grid_mass), the
checker of the GPU's deterministic P2G mode, pinned against a plain Python
restatement of the same order: for every node n, the 27 base cells
n - (i, j, k) with (i, j, k) in lexicographic order, each cell's particles by
ascending index, w = N(n_x - x/dx) N(n_y - y/dx) N(n_z - z/dx) with the
reference's quadratic kernel (rust/crates/cpu/src/kernels.rs:17-26) and the
sum of w m taken left to right -- every operation a single fp32 rounding,
which numpy float32 scalars reproduce.  The base cell is
floor(x/dx - 1/2) (kernels.rs:46-49); tombstoned particles take no part."""

import numpy as np

from oracle import oracle as om

F32 = np.float32
TOMBSTONED = 1 << 5  # ParticleFlags bit of the reference (file_frame/src/particles.rs:21-33)


def kernel(r):
    r = abs(r)
    if r < F32(0.5):
        return F32(0.75) - r * r
    if r < F32(1.5):
        t = F32(1.5) - r
        return F32(0.5) * t * t
    return F32(0.0)


def restated(pos, mass, flags, dx):
    dx = F32(dx)
    cells = {}
    for p in range(len(mass)):
        if flags[p] & TOMBSTONED:
            continue
        c = tuple(int(np.floor(F32(pos[p, a]) / dx - F32(0.5))) for a in range(3))
        cells.setdefault(c, []).append(p)
    nodes = sorted({(c[0] + i, c[1] + j, c[2] + k) for c in cells for i in range(3) for j in range(3)
                    for k in range(3)})
    ids, out = [], []
    for nd in nodes:
        s = F32(0.0)
        for i in range(3):
            for j in range(3):
                for k in range(3):
                    for p in cells.get((nd[0] - i, nd[1] - j, nd[2] - k), ()):
                        w = F32(1.0)
                        for a in range(3):
                            r = F32(nd[a]) - F32(pos[p, a]) / dx
                            w = kernel(r) if a == 0 else w * kernel(r)
                        s = s + w * F32(mass[p])
        if s > 0:
            ids.append(nd)
            out.append(s)
    return np.array(ids, np.int32).reshape(-1, 3), np.array(out, np.float32)


def test_deterministic_mass_matches_its_restatement():
    rng = np.random.default_rng(11)
    n = 300
    dx = 1.0 / 64
    # clustered so that cells hold several particles and nodes many contributions
    pos = (0.3 + 0.06 * rng.random((n, 3))).astype(np.float32)
    mass = rng.uniform(0.5, 2.0, n).astype(np.float32) * np.float32(1e-4)
    flags = np.ones(n, np.uint32)
    flags[rng.choice(n, 20, replace=False)] |= TOMBSTONED
    ids, m = om.deterministic_grid_mass(pos, mass, flags, dx)
    ids_r, m_r = restated(pos, mass, flags, dx)
    np.testing.assert_array_equal(ids, ids_r)
    np.testing.assert_array_equal(m.view(np.uint32), m_r.view(np.uint32))
    # and it conserves mass to fp32 rounding
    live = mass[(flags & TOMBSTONED) == 0].astype(np.float64).sum()
    assert abs(float(m.astype(np.float64).sum()) - float(live)) <= 1e-5 * float(mass.sum())
