"""Served evaluation (gwn_server): resident meshes, continuous batching,
HBM-budget admission with LRU eviction.

Every served result is compared with the single-mesh path
(FastWindingNumberBVH.eval, i.e. gwn_soup_eval) on the same mesh and
queries, and with itself alone vs. in a mix of concurrent requests.  The walk
of one query does not depend on the other queries of its warp or batch, so
the stated tolerance for both comparisons is 1e-12 (in practice the results
are bitwise equal)."""
import threading

import numpy as np
import pytest

from libigl_gb300 import synth

TOL_SAME = 1e-12


def _meshes(count, seed=11):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        nu = int(rng.integers(7, 30))
        V, F = synth.geodesic_sphere(nu)
        V = synth.sh_deform(V, rng)
        if k % 3 == 1:
            F = synth.delete_patch(F, rng, max(1, F.shape[0] // 50))
        out.append((V, F))
    return out


def _queries(V, n, seed, dtype=np.float32):
    rng = np.random.default_rng(seed)
    lo, hi = V.min(0), V.max(0)
    Q = rng.uniform(lo, hi, size=(n, 3))
    # a share of near-surface queries exercises the FP64 near field and the
    # threshold re-evaluation
    m = n // 5
    idx = rng.integers(V.shape[0], size=m)
    Q[:m] = V[idx] * (1.0 + rng.choice([-1, 1], size=(m, 1)) * 10.0 ** rng.uniform(-6, -2, (m, 1)))
    return Q.astype(dtype)


@pytest.mark.gpu
def test_served_equals_single_mesh_path(cuda):
    import libigl_gb300 as G
    meshes = _meshes(4)
    with G.Server(hbm_budget_bytes=8 << 30, max_batch_queries=1 << 20, slots=2) as S:
        ids = [S.add_mesh(V, F) for V, F in meshes]
        for prec in ("mixed", "fp64"):
            for k, ((V, F), mid) in enumerate(zip(meshes, ids)):
                for qdt in (np.float32, np.float64):
                    Q = _queries(V, 5000 + 371 * k, seed=100 + k, dtype=qdt)
                    W, lat = S.submit(mid, Q, 2.0, prec, out_dtype=np.float64).wait(60)
                    bvh = G.FastWindingNumberBVH(V, F, 2)
                    Wr = bvh.eval(Q, 2.0, prec, out_dtype=np.float64)
                    bvh.close()
                    assert lat > 0
                    assert np.all(np.isfinite(W))
                    assert np.abs(W - Wr).max() <= TOL_SAME, (prec, k, qdt)
        st = S.stats()
        assert st["builds"] == 4 and st["evictions"] == 0
        assert st["requests_done"] == 16 and st["kernels_per_batch"] > 0


@pytest.mark.gpu
def test_alone_and_in_the_mix_agree(cuda):
    """Each request evaluated alone (idle server) and again among many
    concurrent requests on other meshes gives the same result."""
    import libigl_gb300 as G
    meshes = _meshes(6, seed=12)
    rng = np.random.default_rng(5)
    reqs = []
    for i in range(48):
        k = int(rng.integers(len(meshes)))
        n = int(np.exp(rng.uniform(np.log(50), np.log(40000))))
        reqs.append((k, _queries(meshes[k][0], n, seed=1000 + i),
                     "mixed" if i % 4 else "fp64"))
    with G.Server(hbm_budget_bytes=8 << 30, max_batch_queries=1 << 18, slots=3) as S:
        ids = [S.add_mesh(V, F) for V, F in meshes]
        alone = []
        for k, Q, prec in reqs:
            W, _ = S.submit(ids[k], Q, 2.0, prec, np.float64).wait(60)
            alone.append(W.copy())
        b0 = S.stats()["batches"]
        mixed = [None] * len(reqs)

        def client(part):
            subs = [(i, S.submit(ids[reqs[i][0]], reqs[i][1], 2.0, reqs[i][2], np.float64))
                    for i in part]
            for i, r in subs:
                mixed[i] = r.wait(120)[0]
        parts = [list(range(t, len(reqs), 4)) for t in range(4)]
        th = [threading.Thread(target=client, args=(p,)) for p in parts]
        for t in th:
            t.start()
        for t in th:
            t.join()
        st = S.stats()
        # the mix was batched: fewer batches than requests
        assert st["batches"] - b0 < len(reqs)
    for a, m in zip(alone, mixed):
        assert m is not None
        assert np.abs(a - m).max() <= TOL_SAME


@pytest.mark.gpu
def test_lru_eviction_under_a_small_budget(cuda):
    import libigl_gb300 as G
    meshes = _meshes(4, seed=13)
    sizes = [F.shape[0] for _, F in meshes]
    # room for about two of the largest trees (as built by the server: the
    # default tree of FastWindingNumberBVH)
    Vb, Fb = meshes[int(np.argmax(sizes))]
    big = G.FastWindingNumberBVH(Vb, Fb, 2)
    budget = int(2.2 * big.stats["device_bytes"])
    big.close()
    with G.Server(hbm_budget_bytes=budget, max_batch_queries=1 << 16, slots=2) as S:
        ids = [S.add_mesh(V, F) for V, F in meshes]
        refs = []
        for k, (V, F) in enumerate(meshes):
            Q = _queries(V, 3000, seed=7 + k)
            bvh = G.FastWindingNumberBVH(V, F, 2)
            refs.append((Q, bvh.eval(Q, 2.0, "mixed", out_dtype=np.float64)))
            bvh.close()
        for rnd in range(3):
            for k in range(len(meshes)):
                Q, Wr = refs[k]
                W, _ = S.submit(ids[k], Q, 2.0, "mixed", np.float64).wait(60)
                assert np.abs(W - Wr).max() <= TOL_SAME
        st = S.stats()
        assert st["evictions"] > 0
        assert st["builds"] > 4  # evicted trees were rebuilt on their next request
        assert st["resident_bytes"] <= budget
        assert st["peak_resident_bytes"] <= budget


@pytest.mark.gpu
def test_server_errors(cuda):
    import libigl_gb300 as G
    from libigl_gb300 import GwnError
    V, F = synth.geodesic_sphere(20)
    with G.Server(hbm_budget_bytes=1 << 20, max_batch_queries=1024, slots=1) as S:
        mid = S.add_mesh(V, F)
        # more than the budget: the request fails, the server keeps serving
        with pytest.raises(GwnError):
            S.submit(mid, np.zeros((10, 3), np.float32)).wait(60)
        small = S.add_mesh(*synth.geodesic_sphere(1))
        W, _ = S.submit(small, np.zeros((5, 3), np.float32), 2.0, "mixed", np.float64).wait(60)
        assert np.allclose(W, 1.0, atol=1e-6)
        # empty request, capacity limit, unknown mesh
        W, _ = S.submit(small, np.zeros((0, 3), np.float32)).wait(10)
        assert W.shape == (0,)
        with pytest.raises(GwnError):
            S.submit(small, np.zeros((1025, 3), np.float32))
        with pytest.raises(GwnError):
            S.submit(12345, np.zeros((3, 3), np.float32))
        S.remove_mesh(small)
        with pytest.raises(GwnError):
            S.submit(small, np.zeros((3, 3), np.float32))


@pytest.mark.gpu
def test_cold_build_does_not_block_resident_meshes(cuda):
    """A request whose mesh is not resident waits for its tree, which builds
    on the server's builder thread; requests for resident meshes submitted
    after it keep being batched and finish first.  Every result still equals
    the single-mesh path."""
    import time
    import libigl_gb300 as G
    rng = np.random.default_rng(21)
    Vb, Fb = synth.icosphere(8)  # 1.3M triangles: a build of tens of ms
    Vb = synth.sh_deform(Vb, rng)
    small = _meshes(2, seed=23)
    with G.Server(hbm_budget_bytes=16 << 30, max_batch_queries=1 << 18, slots=2) as S:
        sid = [S.add_mesh(V, F) for V, F in small]
        for k, (V, _) in enumerate(small):  # make the small meshes resident
            S.submit(sid[k], _queries(V, 64, seed=5 + k)).wait(60)
        bid = S.add_mesh(Vb, Fb)
        builds0 = S.stats()["builds"]
        Qb = _queries(Vb, 2000, seed=31)
        t_big = time.perf_counter()
        big = S.submit(bid, Qb, 2.0, "mixed", np.float64)
        subs = []
        for i in range(16):
            k = i % 2
            Q = _queries(small[k][0], 500, seed=40 + i)
            subs.append((k, Q, time.perf_counter(), S.submit(sid[k], Q, 2.0, "mixed", np.float64)))
        done_small = []
        for k, Q, t0, r in subs:
            W, lat = r.wait(60)
            done_small.append(t0 + lat)
            bvh = G.FastWindingNumberBVH(*small[k], 2)
            assert np.abs(W - bvh.eval(Q, 2.0, "mixed", out_dtype=np.float64)).max() <= TOL_SAME
            bvh.close()
        Wb, lat_b = big.wait(120)
        assert S.stats()["builds"] == builds0 + 1
        # the small requests did not wait for the build
        assert max(done_small) < t_big + lat_b
        bvh = G.FastWindingNumberBVH(Vb, Fb, 2)
        assert np.abs(Wb - bvh.eval(Qb, 2.0, "mixed", out_dtype=np.float64)).max() <= TOL_SAME
        bvh.close()
