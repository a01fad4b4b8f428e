"""Known-answer tests of the CPU oracle (no GPU).

The reference ships no tests or golden vectors, so the oracle is pinned here
to hand-derived answers of the reference's own rules (Bresenham walk of
dyn_calc_kernel, periodic D / D^T, shrinkage, b scaling, ray-list order), to
analytic Siddon lengths, and to an independent numpy restatement of the loop.
"""
import math

import numpy as np
import pytest

from tval3_gb300.api import Geometry


def bres_python(s, e):
    """The reference loop, 3d/tval3_gpu_3d_kernels.cu:1649-1763, in Python."""
    x, y, z = s
    out = [(x, y, z)]
    d1, d2, d3 = e[0] - x, e[1] - y, e[2] - z
    m1, m2, m3 = abs(d1), abs(d2), abs(d3)
    if m1 >= m2 and m1 >= m3:
        order = (0, 1, 2)
    elif m2 >= m1 and m2 >= m3:
        d1, d2 = d2, d1
        order = (1, 0, 2)
    else:
        d1, d3, d2 = d3, d2, d1
        order = (2, 0, 1)
    p = [x, y, z]
    inc = [-1 if d < 0 else 1 for d in (d1, d2, d3)]
    m1, m2, m3 = abs(d1), abs(d2), abs(d3)
    e1, e2 = 2 * m2 - m1, 2 * m3 - m1
    for _ in range(m1):
        if e1 > 0:
            p[order[1]] += inc[1]
            e1 -= 2 * m1
        if e2 > 0:
            p[order[2]] += inc[2]
            e2 -= 2 * m1
        e1 += 2 * m2
        e2 += 2 * m3
        p[order[0]] += inc[0]
        out.append(tuple(p))
    return out


def bres_closed_form(s, e):
    """The closed form used by the device traversal: s(j) = (2 m j + m1 - 1) // (2 m1)."""
    d = [e[a] - s[a] for a in range(3)]
    m = [abs(v) for v in d]
    if m[0] >= m[1] and m[0] >= m[2]:
        a1, a2, a3 = 0, 1, 2
    elif m[1] >= m[0] and m[1] >= m[2]:
        a1, a2, a3 = 1, 0, 2
    else:
        a1, a2, a3 = 2, 0, 1
    m1 = m[a1]
    out = []
    for j in range(m1 + 1):
        c = list(s)
        c[a1] = s[a1] + (1 if d[a1] >= 0 else -1) * j
        for a in (a2, a3):
            k = (2 * m[a] * j + m1 - 1) // (2 * m1) if m1 else 0
            c[a] = s[a] + (1 if d[a] >= 0 else -1) * k
        out.append(tuple(c))
    return out


# hand-enumerated walks (x, y, z), derived step by step from the reference loop
BRES_KAT = [
    ((0, 0, 0), (3, 0, 0), [(0, 0, 0), (1, 0, 0), (2, 0, 0), (3, 0, 0)]),
    ((0, 0, 0), (2, 2, 2), [(0, 0, 0), (1, 1, 1), (2, 2, 2)]),
    ((0, 0, 0), (4, 1, 0), [(0, 0, 0), (1, 0, 0), (2, 0, 0), (3, 1, 0), (4, 1, 0)]),
    ((2, 5, 1), (1, 0, 0), [(2, 5, 1), (2, 4, 1), (2, 3, 1), (1, 2, 0), (1, 1, 0), (1, 0, 0)]),
    ((0, 0, 0), (1, 2, 3), [(0, 0, 0), (0, 1, 1), (1, 1, 2), (1, 2, 3)]),
    ((1, 1, 1), (1, 1, 1), [(1, 1, 1)]),
]


@pytest.mark.parametrize("s,e,walk", BRES_KAT)
def test_bresenham_hand_walks(s, e, walk, oracle):
    assert bres_python(s, e) == walk
    assert bres_closed_form(s, e) == walk
    g = Geometry(rv_x=6, rv_y=6, rv_z=6, x_emitters=[s[0]], y_emitters=[s[1]], z_emitters=[s[2]],
                 x_receivers=[e[0]], y_receivers=[e[1]], z_receivers=[e[2]])
    ptr, ind, val = oracle.bresenham_csr(g)
    assert ptr.tolist() == [0, len(walk)]
    assert ind.tolist() == [z * 36 + x * 6 + y for (x, y, z) in walk]
    assert np.all(val == 1.0)


def test_bresenham_closed_form_exhaustive():
    rng = np.random.default_rng(1)
    for _ in range(3000):
        s = tuple(int(v) for v in rng.integers(0, 40, 3))
        e = tuple(int(v) for v in rng.integers(0, 40, 3))
        assert bres_closed_form(s, e) == bres_python(s, e)


def test_bresenham_endpoint_outside_rejected(oracle):
    g = Geometry(rv_x=4, rv_y=4, rv_z=4, x_emitters=[0], y_emitters=[0], z_emitters=[0],
                 x_receivers=[4], y_receivers=[0], z_receivers=[0])
    with pytest.raises(ValueError):
        oracle.bresenham_csr(g)


def test_ray_list_order(oracle):
    # 3d/mat_vec_mul_dynamic.h:531-536: emitter i // R, receiver (i // (E*R)) * R + i % R
    E, R, M = 3, 4, 2
    use = np.array([1, 0, 1, 1, 0, 0, 1, 0, 1, 1, 1, 0], np.uint32)
    pairs = oracle.ray_list(M, E, R, use)
    exp = [(i // R, (i // (E * R)) * R + i % R) for i in range(M * E * R) if use[i % (E * R)]]
    assert [tuple(p) for p in pairs.tolist()] == exp
    g = Geometry(rv_x=2, rv_y=2, rv_z=2, x_emitters=np.zeros(6), y_emitters=np.zeros(6), z_emitters=np.zeros(6),
                 x_receivers=np.zeros(8), y_receivers=np.zeros(8), z_receivers=np.zeros(8), num_emitters=3,
                 num_receivers=4, numMPs=2, use_path=use)
    assert [tuple(p) for p in g.ray_pairs().tolist()] == exp


def _siddon_one(oracle, p0, p1, dims, scale=1.0):
    g = Geometry(rv_x=dims[0], rv_y=dims[1], rv_z=dims[2], x_emitters=[0], y_emitters=[0], z_emitters=[0],
                 x_receivers=[0], y_receivers=[0], z_receivers=[0], scale_factor=scale, traversal=1,
                 pos=([p0[0]], [p0[1]], [p0[2]], [p1[0]], [p1[1]], [p1[2]]))
    ptr, ind, val = oracle.siddon_csr(g)
    return ind.tolist(), val.astype(np.float64)


def test_siddon_axis_aligned(oracle):
    ind, val = _siddon_one(oracle, (-1.0, 1.5, 0.5), (5.0, 1.5, 0.5), (4, 4, 1))
    assert ind == [x * 4 + 1 for x in range(4)]
    assert np.allclose(val, 1.0, rtol=0, atol=1e-7)


def test_siddon_diagonal_through_corner(oracle):
    ind, val = _siddon_one(oracle, (0.0, 0.0, 0.5), (2.0, 2.0, 0.5), (4, 4, 1))
    assert ind == [0, 1 * 4 + 1]
    assert np.allclose(val, math.sqrt(2.0), rtol=1e-7)


def test_siddon_slope_half(oracle):
    ind, val = _siddon_one(oracle, (0.5, 0.5, 0.5), (2.5, 1.5, 0.5), (4, 4, 1), scale=2.0)
    assert ind == [0, 4, 5, 9]
    assert np.allclose(val, 2.0 * 0.25 * math.sqrt(5.0), rtol=1e-7)


def test_siddon_outside_is_empty(oracle):
    ind, _ = _siddon_one(oracle, (-1.0, -1.0, 0.5), (-1.0, 5.0, 0.5), (4, 4, 1))
    assert ind == []


def _siddon_reference_numpy(p0, p1, dims):
    """Classic Siddon (all plane crossings, sorted, midpoints) in numpy."""
    p0, p1 = np.array(p0, float), np.array(p1, float)
    d = p1 - p0
    L = np.linalg.norm(d)
    ts = [0.0, 1.0]
    for a in range(3):
        if d[a] != 0:
            ks = np.arange(0, dims[a] + 1)
            t = (ks - p0[a]) / d[a]
            ts += list(t[(t > 0) & (t < 1)])
    ts = np.unique(ts)
    out = {}
    for t0, t1 in zip(ts[:-1], ts[1:]):
        mid = p0 + 0.5 * (t0 + t1) * d
        if np.all(mid >= 0) and np.all(mid < dims):
            ix, iy, iz = np.floor(mid).astype(int)
            k = iz * dims[0] * dims[1] + ix * dims[1] + iy
            out[k] = out.get(k, 0.0) + (t1 - t0) * L
    return out


def test_siddon_random_rays_vs_classic(oracle):
    rng = np.random.default_rng(3)
    dims = (7, 5, 6)
    for _ in range(200):
        p0 = rng.uniform(-2, 9, 3)
        p1 = rng.uniform(-2, 9, 3)
        ind, val = _siddon_one(oracle, p0, p1, dims)
        ref = _siddon_reference_numpy(p0, p1, dims)
        got = {}
        for k, v in zip(ind, val):
            got[k] = got.get(k, 0.0) + v
        assert set(got) == set(k for k, v in ref.items() if v > 1e-9)
        for k in got:
            assert abs(got[k] - ref[k]) <= 1e-5 * max(1.0, ref[k])


def test_siddon_length_sum_is_chord(oracle):
    rng = np.random.default_rng(4)
    dims = (9, 8, 7)
    for _ in range(100):
        p0 = rng.uniform(0, 1, 3) * dims
        p1 = rng.uniform(0, 1, 3) * dims
        _, val = _siddon_one(oracle, p0, p1, dims)
        assert abs(val.sum() - np.linalg.norm(p1 - p0)) < 1e-5 * max(1.0, np.linalg.norm(p1 - p0))


def test_D_Dt_periodic_kat(oracle):
    U = np.array([1.0, 2.0, 4.0])  # p = 3 (y), q = r = 1
    DU = oracle.D(U, (3, 1, 1))
    assert DU[0].tolist() == [1.0, 2.0, -3.0]
    assert DU[1].tolist() == [0.0, 0.0, 0.0] and DU[2].tolist() == [0.0, 0.0, 0.0]
    out = oracle.Dt(np.stack([DU[0], np.zeros(3), np.zeros(3)]), (3, 1, 1))
    assert out.tolist() == [-4.0, -1.0, 5.0]


def test_D_matches_roll_and_adjoint(oracle):
    rng = np.random.default_rng(5)
    p, q, r = 5, 4, 3
    U = rng.normal(size=(r, q, p))
    DU = oracle.D(U, (p, q, r))
    ref = np.stack([np.roll(U, -1, 2) - U, np.roll(U, -1, 1) - U, np.roll(U, -1, 0) - U]).reshape(3, -1)
    assert np.array_equal(DU, ref)
    P = rng.normal(size=(3, p * q * r))
    lhs = np.sum(DU * P)
    rhs = np.dot(U.reshape(-1), oracle.Dt(P, (p, q, r)))
    assert abs(lhs - rhs) < 1e-12 * max(1.0, abs(lhs))


def test_shrinkage_closed_forms(oracle):
    DU = np.array([[1.0], [-0.2], [-2.0]])
    W, lam1 = oracle.shrink(DU, np.zeros_like(DU), 2.0, iso=False)
    assert W.reshape(-1).tolist() == [0.5, 0.0, -1.5] and lam1 == 2.0
    DU = np.array([[3.0], [4.0], [0.0]])
    W, lam1 = oracle.shrink(DU, np.zeros_like(DU), 2.0, iso=True)
    assert np.allclose(W.reshape(-1), [2.7, 3.6, 0.0]) and abs(lam1 - 4.5) < 1e-12
    W, lam1 = oracle.shrink(np.zeros((3, 1)), np.zeros((3, 1)), 2.0, iso=True)
    assert np.all(W == 0) and lam1 == 0.0


def test_transpose_and_spmv(oracle):
    import scipy.sparse as sp
    rng = np.random.default_rng(6)
    A = sp.random(40, 30, density=0.2, random_state=7, format="csr", dtype=np.float32)
    ptr, ind, val = A.indptr.astype(np.int32), A.indices.astype(np.int32), A.data.astype(np.float32)
    tptr, tind, tval = oracle.transpose(40, 30, ptr, ind, val)
    At = A.T.tocsr()
    At.sort_indices()
    assert np.array_equal(tptr, At.indptr) and np.array_equal(tind, At.indices) and np.array_equal(tval, At.data)
    x = rng.normal(size=30)
    assert np.allclose(oracle.spmv(ptr, ind, val, x), A.astype(np.float64) @ x, rtol=1e-12)


def test_oracle_matches_numpy_restatement(oracle):
    import scipy.sparse as sp
    from tests import np_tval3
    from tval3_gb300 import workloads as W
    geo = W.ring_geometry(16, 24)
    x = W.ellipse_phantom(16, 3, seed=2, axes=(2.0, 6.0))
    ptr, ind, val = oracle.siddon_csr(geo)
    A = sp.csr_matrix((val.astype(np.float64), ind, ptr), shape=(ptr.size - 1, x.size))
    b = W.add_noise(A @ x.reshape(-1).astype(np.float64), 0.01, 0).astype(np.float64)
    for iso in (0, 1):
        o = dict(mu=256., mu0=64., beta=32., beta0=8., rate_cnt=2., tol=1e-4, tol_inn=1e-3, maxcnt=10, maxit=25,
                 c=1e-5, gamma=0.6, gam=0.9995, rate_gam=0.9, nonneg=1)
        Unp, inf = np_tval3.tval3(A, b, (16, 16, 1), o, iso=bool(iso))
        Uor, io = oracle.tval3_csr((16, 16, 1), ptr, ind, val, b, dict(o, tv_type=iso), prec=0)
        assert (inf["total"], inf["outer"], inf["bt"], inf["rs"]) == \
            (io["total_iters"], io["outer_iters"], io["backtracks"], io["restarts"])
        assert np.linalg.norm(Unp - Uor.reshape(-1)) <= 1e-9 * np.linalg.norm(Uor)


def test_scale_b_rules(oracle):
    # scaleb_gpu (3d/tval3_gpu_3d.cpp:226-266): dif = |b[argmax|b|] - b[argmin|b|]|
    import ctypes as C
    from oracle.oracle import OracleInfo
    ptr = np.array([0, 1, 2], np.int32)
    ind = np.array([0, 1], np.int32)
    val = np.array([1.0, 1.0], np.float32)
    for b, scl in (([0.1, 0.2], 0.5 / 0.1), ([1.0, 3.0], 1.5 / 2.0), ([0.0, 1.0], 1.0), ([0.5, 0.5], 1.0)):
        _, info = oracle.tval3_csr((2, 1, 1), ptr, ind, val, np.array(b), dict(maxit=1, maxcnt=1), prec=0)
        assert abs(info["scl"] - scl) < 1e-12


def test_oracle_layers_of_identical_columns_equal_single_solve(oracle):
    """A joint solve of L identical layers takes the same steps as the single
    solve (every inner product, f and the Armijo terms scale by L), so each
    layer equals the single-layer solution."""
    from tval3_gb300 import workloads as W
    geo = W.ring_geometry(16, 24)
    x = W.ellipse_phantom(16, 3, seed=1, axes=(2.0, 6.4))
    ptr, ind, val = oracle.siddon_csr(geo)
    b = W.add_noise(oracle.spmv(ptr, ind, val, x), 0.01, 1).astype(np.float64)
    o = dict(mu=256., mu0=64., beta=32., beta0=8., tol=1e-4, maxit=60, tv_iso=0)
    U1, i1 = oracle.tval3_csr((16, 16, 1), ptr, ind, val, b, o)
    UL, iL = oracle.tval3_layers((16, 16, 1), 3, (ptr, ind, val), np.concatenate([b, b, b]), o)
    assert (iL["total_iters"], iL["outer_iters"], iL["backtracks"]) == \
        (i1["total_iters"], i1["outer_iters"], i1["backtracks"])
    for l in range(3):
        assert np.linalg.norm(UL[l].reshape(-1) - U1.reshape(-1)) <= 1e-9 * np.linalg.norm(U1)


def test_oracle_skip_heuristic(oracle):
    """The skip-A^T rule of get_g_gpu (3d/tval3_gpu_3d.cpp:398-468):
    ratio 0 forms A^T Au in every get_g (1 at start-up + one per iteration +
    one per restart); maxRelativeChange 0 forces every product, so the solve
    is identical to the exact one; a small maxRelativeChange lets the budget
    skip a few products.  (Skipped products leave the Barzilai-Borwein step
    without its A^T A curvature, so larger thresholds make the loop unstable
    on this problem, in the reference's rule as here.)"""
    from tval3_gb300 import workloads as W
    geo = W.ring_geometry(16, 24)
    x = W.ellipse_phantom(16, 3, seed=1, axes=(2.0, 6.4))
    ptr, ind, val = oracle.siddon_csr(geo)
    b = W.add_noise(oracle.spmv(ptr, ind, val, x), 0.01, 1).astype(np.float64)
    o = dict(mu=256., mu0=64., beta=32., beta0=8., tol=1e-4, maxit=80, tv_iso=0)
    U0, i0 = oracle.tval3_csr((16, 16, 1), ptr, ind, val, b, o)
    assert i0["products_T"] == 1 + i0["total_iters"] + i0["restarts"]
    U1, i1 = oracle.tval3_csr((16, 16, 1), ptr, ind, val, b, dict(o, skipMulRatio=0.5, maxRelativeChange=0.0))
    assert np.array_equal(U1, U0) and i1["total_iters"] == i0["total_iters"]
    U2, i2 = oracle.tval3_csr((16, 16, 1), ptr, ind, val, b,
                              dict(o, skipMulRatio=0.5, numInitIterations=4, maxRelativeChange=1e-3))
    assert i2["products_T"] < 1 + i2["total_iters"] + i2["restarts"]
    assert np.linalg.norm(U2 - U0) < 0.3 * np.linalg.norm(U0)
