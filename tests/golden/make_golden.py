"""Generate the committed golden fixtures from the reference's own code.

Run where the libigl reference tree is available (the reference soup code is
compiled from it into oracle/_ref/ by oracle/build_ref.sh):

    GWN_REFERENCE_ROOT=<libigl source tree> python tests/golden/make_golden.py

Writes tests/golden/soup_reference.npz: for a handful of seeded meshes
(single triangle, four triangles, a deformed icosphere with holes, a random
soup) and seeded query sets, the reference's UT_SolidAngle winding numbers
(order 2, accuracy_scale 2, FP32 inside, exactly as
include/igl/fast_winding_number.cpp:383-437 calls it) and the exact FP64
winding numbers (brute-force oracle) for the same queries; and for every
mesh the reference's own UT_BVH<4> node array (<name>/tree: 4 lanes per
node, exported from the compiled reference), including three meshes chosen
for their trees (ties on a grid, nodes of more than 1024 boxes, degenerate
and repeated triangles).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from libigl_gb300 import synth  # noqa: E402
from oracle import oracle as O  # noqa: E402


def cases():
    rng = np.random.default_rng(1234)
    out = {}
    # one triangle: the reference tree is a single node with one item child
    V = np.array([[0.0, 0.0, 0.0], [1.0, 0.2, 0.1], [0.3, 0.9, -0.2]])
    F = np.array([[0, 1, 2]], np.int32)
    out["one_tri"] = (V, F)
    # four triangles: one node, four item children (tree identical to any 4-leaf grouping
    # at the level of evaluated moments)
    V = rng.normal(size=(12, 3))
    F = np.arange(12, dtype=np.int32).reshape(4, 3)
    out["four_tris"] = (V, F)
    # deformed icosphere subdiv 3 with 3% faces deleted (holes -> fractional W)
    V, F = synth.icosphere(3)
    V = synth.sh_deform(V, rng)
    F = synth.delete_random_faces(F, rng, 0.03)
    out["sphere_holes"] = (V, F.astype(np.int32))
    # a closed icosphere subdiv 4 (5120 tris)
    V, F = synth.icosphere(4)
    V = V * (1.0 + rng.normal(0, 0.02, V.shape[0]))[:, None]
    out["sphere_closed"] = (V, F)
    # random soup
    V = rng.uniform(-1, 1, size=(300, 3))
    F = rng.integers(0, 300, size=(100, 3)).astype(np.int32)
    out["random_soup"] = (V, F)
    return out


def tree_cases():
    """Meshes whose trees exercise every split of UT_BVH<4>: exact ties
    (a flat grid), nodes of more than 1024 boxes (span splits and their
    partitions), and degenerate boxes."""
    rng = np.random.default_rng(4321)
    out = {}
    # deformed icosphere subdiv 5 with 1% of its faces deleted (20,275 tris)
    V, F = synth.icosphere(5)
    V = synth.sh_deform(V, rng)
    F = synth.delete_random_faces(F, rng, 0.01)
    out["sphere5_holes"] = (V, F.astype(np.int32))
    # a flat 40 x 40 grid of squares (many equal centres)
    g = np.stack(np.meshgrid(np.arange(41.0), np.arange(41.0), [0.0], indexing="ij"),
                 -1).reshape(-1, 3)
    F = []
    for i in range(40):
        for j in range(40):
            a = i * 41 + j
            F += [[a, a + 1, a + 41], [a + 1, a + 42, a + 41]]
    out["grid40"] = (g, np.array(F, np.int32))
    # a soup with repeated and zero-area triangles
    V = rng.normal(size=(500, 3))
    F = rng.integers(0, 500, size=(3000, 3))
    F[::7] = F[::7, [0, 0, 1]]          # two equal corners: zero area
    F[1::11] = F[0:-1:11][: len(F[1::11])]  # repeats of other triangles
    out["degenerate_soup"] = (V, F.astype(np.int32))
    return out


def queries(V, F, rng, n=2000):
    lo, hi = V.min(0), V.max(0)
    c, h = (lo + hi) / 2, (hi - lo) / 2 * 1.5 + 1e-3
    far = c + rng.uniform(-1, 1, size=(n // 2, 3)) * h
    # near-surface queries on faces of non-zero area: a point on a zero-area
    # triangle lies exactly on the surface, where W is not defined
    area = np.linalg.norm(np.cross(V[F[:, 1]] - V[F[:, 0]], V[F[:, 2]] - V[F[:, 0]]), axis=1)
    Fs = F[area > 0]
    P, f = synth.sample_on_faces(V, Fs, rng, n - n // 2)
    nrm = synth.face_normals(V, Fs[f])
    d = 10.0 ** rng.uniform(-4, -1, size=P.shape[0]) * rng.choice([-1.0, 1.0], P.shape[0])
    return np.concatenate([far, P + nrm * d[:, None]])


def main():
    if O.build_ref() is None:
        raise SystemExit("reference tree not available (set GWN_REFERENCE_ROOT to the libigl "
                         "source tree): cannot build oracle/_ref")
    rng = np.random.default_rng(99)
    arrays = {}
    for name, (V, F) in cases().items():
        Q = queries(V, F, rng)
        ref = O.RefSoup(V, F, order=2)
        Wref = ref.eval(Q, 2.0)
        Wex = O.winding_number(V, F, Q)
        arrays[f"{name}/V"] = V
        arrays[f"{name}/F"] = F
        arrays[f"{name}/Q"] = Q
        arrays[f"{name}/W_ref"] = Wref
        arrays[f"{name}/W_exact"] = Wex
        arrays[f"{name}/tree"] = ref.tree()
        print(f"{name}: {F.shape[0]} tris, {Q.shape[0]} queries, "
              f"max|ref-exact| = {np.abs(Wref - Wex).max():.3e}")
    # the reference's own trees (UT_BVH<4> node arrays) and values on meshes
    # that reach every kind of split
    for name, (V, F) in tree_cases().items():
        Q = queries(V, F, rng, n=4000)
        ref = O.RefSoup(V, F, order=2)
        arrays[f"{name}/V"] = V
        arrays[f"{name}/F"] = F
        arrays[f"{name}/Q"] = Q
        arrays[f"{name}/W_ref"] = ref.eval(Q, 2.0)
        arrays[f"{name}/tree"] = ref.tree()
        print(f"{name}: {F.shape[0]} tris, {ref.tree().shape[0]} nodes")
    np.savez_compressed(os.path.join(HERE, "soup_reference.npz"), **arrays)


if __name__ == "__main__":
    main()
