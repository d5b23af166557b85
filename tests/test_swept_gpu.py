"""igl::swept_volume_signed_distance and igl::flood_fill on the GPU against
their CPU restatements (oracle/swept.cpp, oracle.swept_volume_signed_distance,
which follows include/igl/swept_volume_signed_distance.cpp:21-160 over the
oracle's AABB, exact winding number, soup code and pseudonormal test).

Tolerances: flood fill bit-exact; unsigned and winding-number types 1e-12
relative + 1e-13 (distances from the same closest-point formula, W exact);
pseudonormal exact except at points whose closest feature is shared (the
closest triangle of a tie is the first found); fast winding number within
the soup approximation (the GPU tree differs from the reference's, and the
reference evaluates on the float copy of V): |dS| <= 1e-2 |S| + 1e-6 with
the same sign wherever |s| > 0.05.
"""
import numpy as np
import pytest

import libigl_gb300 as G
from libigl_gb300 import synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _mesh():
    V, F = synth.icosphere(2)
    rng = np.random.default_rng(41)
    V = synth.sh_deform(V, rng, lmax=4, sigma=0.08) * np.array([1.0, 0.6, 0.4])
    return np.ascontiguousarray(V), np.ascontiguousarray(F, dtype=np.int32)


def _rot(axis, ang):
    axis = np.asarray(axis, float) / np.linalg.norm(axis)
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    return np.eye(3) + np.sin(ang) * K + (1 - np.cos(ang)) * K @ K


def _sweep(nT=6):
    T = []
    for k in range(nT):
        u = k / max(nT - 1, 1)
        A = np.zeros((3, 4))
        A[:, :3] = _rot([0.3, 1.0, 0.2], 1.2 * u)
        A[:, 3] = [1.5 * u, 0.4 * np.sin(3 * u), 0.2 * u]
        T.append(A)
    return np.array(T)


def _grid(res, lo, hi):
    xs = [np.linspace(lo[d], hi[d], res[d]) for d in range(3)]
    h = float(xs[0][1] - xs[0][0])
    Z, Y, X = np.meshgrid(xs[2], xs[1], xs[0], indexing="ij")
    return np.ascontiguousarray(np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)), h


def _case(res=(26, 18, 14)):
    V, F = _mesh()
    T = _sweep()
    GV, h = _grid(res, [-1.4, -1.3, -1.2], [3.0, 1.5, 1.4])
    return V, F, T, GV, np.array(res, np.int32), h


def _check(S, Sr, sign_type, Smid=None):
    nan = np.isnan(Sr)
    assert np.array_equal(np.isnan(S), nan)
    a, b = S[~nan], Sr[~nan]
    if sign_type in (G.SIGNED_DISTANCE_TYPE_UNSIGNED, G.SIGNED_DISTANCE_TYPE_WINDING_NUMBER,
                     G.SIGNED_DISTANCE_TYPE_DEFAULT):
        np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-13)
    elif sign_type == G.SIGNED_DISTANCE_TYPE_PSEUDONORMAL:
        bad = ~np.isclose(a, b, rtol=1e-12, atol=1e-13)
        assert bad.sum() <= max(2, a.size // 2000), (bad.sum(), a.size)
        np.testing.assert_allclose(np.abs(a[bad]), np.abs(b[bad]), rtol=1e-12, atol=1e-13)
    else:
        assert np.all(np.abs(a - b) <= 1e-2 * np.abs(b) + 1e-6)


@pytest.mark.parametrize("sign_type", [0, 1, 3, 4])
@pytest.mark.parametrize("isolevel", [0.0, np.inf])
def test_swept_volume_matches_oracle(cuda, sign_type, isolevel):
    V, F, T, GV, res, h = _case()
    prec = "mixed" if sign_type == G.SIGNED_DISTANCE_TYPE_FAST_WINDING_NUMBER else "fp64"
    S = G.swept_volume_signed_distance(V, F, T, sign_type, GV, res, h, isolevel, precision=prec)
    Sr = O.swept_volume_signed_distance(V, F, T, sign_type, GV, res, h, isolevel)
    _check(S, Sr, sign_type)
    if np.isfinite(isolevel):
        assert not np.isnan(S).any()  # the flood fill reached everything
    if sign_type != G.SIGNED_DISTANCE_TYPE_UNSIGNED:
        assert (S < 0).any() and (S > 0).any()


def test_swept_volume_seed_and_device(cuda):
    torch = cuda
    V, F, T, GV, res, h = _case()
    S0 = np.random.default_rng(42).uniform(-0.2, 2.0, GV.shape[0])
    S0[::3] = np.nan
    for iso in (0.05, np.inf):
        S = G.swept_volume_signed_distance(V, F, T[:3], 3, GV, res, h, iso, S0=S0)
        Sr = O.swept_volume_signed_distance(V, F, T[:3], 3, GV, res, h, iso, S0=S0)
        _check(S, Sr, 3)
        d = [torch.from_numpy(x).cuda() for x in (V, F, GV, S0)]
        Sd = G.swept_volume_signed_distance(d[0], d[1], T[:3], 3, d[2], res, h, iso, S0=d[3])
        assert np.array_equal(Sd.cpu().numpy(), S, equal_nan=True)


def test_swept_volume_empty(cuda):
    _, _, T, GV, res, h = _case((6, 5, 4))
    V = np.zeros((0, 3))
    F = np.zeros((0, 3), np.int32)
    S = G.swept_volume_signed_distance(V, F, T, 1, GV, res, h, 0.0)
    assert np.isnan(S).all()
    S0 = np.full(GV.shape[0], np.nan)
    S0[17] = 0.25
    S = G.swept_volume_signed_distance(V, F, T, 1, GV, res, h, 0.0, S0=S0)
    assert np.array_equal(S, O.flood_fill(res, S0))


def test_flood_fill_bit_exact(cuda):
    torch = cuda
    rng = np.random.default_rng(43)
    shapes = [(1, 1, 1), (5, 4, 3), (33, 2, 2), (64, 3, 5), (100, 7, 6), (31, 33, 9)]
    for res in shapes:
        n = int(np.prod(res))
        for p in (0.0, 0.003, 0.05, 0.5, 1.0):
            S = np.where(rng.random(n) < p, rng.normal(size=n), np.nan)
            want = O.flood_fill(res, S)
            got = G.flood_fill(res, S.copy())
            assert np.array_equal(got, want, equal_nan=True), (res, p)
            d = torch.from_numpy(S.copy()).cuda()
            G.flood_fill(res, d)
            assert np.array_equal(d.cpu().numpy(), want, equal_nan=True), (res, p)
    # signed cells only in the last sheet / last row
    S = np.full(8 * 6 * 5, np.nan)
    S[-3] = 1.5
    assert np.array_equal(G.flood_fill((8, 6, 5), S.copy()), O.flood_fill((8, 6, 5), S))


def test_swept_volume_mixed_winding_number(cuda):
    """The default (mixed) exact winding-number sign: within 1e-5 relative of
    the FP64 sweep (W within ~1e-6, s = 1 - 2 W) and of the same sign.  With
    a finite isolevel a point whose running minimum sits at the skip
    threshold may be skipped in one run and not the other, so there 99.9% of
    the points must agree."""
    V, F, T, GV, res, h = _case()
    for iso in (np.inf, 0.0):
        Sm = G.swept_volume_signed_distance(V, F, T, 1, GV, res, h, iso)
        S64 = G.swept_volume_signed_distance(V, F, T, 1, GV, res, h, iso, precision="fp64")
        assert np.array_equal(np.isnan(Sm), np.isnan(S64))
        ok = ~np.isnan(S64)
        close = np.abs(Sm[ok] - S64[ok]) <= 1e-5 * np.abs(S64[ok]) + 1e-12
        same = np.sign(Sm[ok]) == np.sign(S64[ok])
        if np.isfinite(iso):
            assert close.mean() >= 0.999 and same.mean() >= 0.999
        else:
            assert close.all() and same.all()
