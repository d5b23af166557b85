"""The reference's "meshes" property test (tests/include/igl/fast_winding_number.cpp:55-107)
on synthetic stand-ins for its data files: for a closed smooth mesh, a closed
lobed mesh and an open hemisphere, the soup fast winding number of the mesh
and the point-cloud fast winding number of its face barycentres (unit face
normals, areas = half the double areas) agree with the exact winding number
at the vertex centroid within 1e-2, the reference's own tolerance.  The CPU
test checks the oracle; the GPU test checks the C-ABI path against both the
exact value and the oracle, plus the exact winding number at the vertices
pulled 20% towards the centroid (tests/include/igl/winding_number.cpp:4-14)."""
import numpy as np
import pytest

from libigl_gb300 import synth
from oracle import oracle as O

TOL_REFERENCE = 1e-2   # test_common::assert_near(..., 1e-2) in the reference test
TOL_MIXED = 1e-4


def _meshes():
    rng = np.random.default_rng(61)
    V, F = synth.geodesic_sphere(30)
    smooth = synth.sh_deform(V, rng, sigma=0.05), F
    lobed = synth.sh_deform(V, rng, lmax=6, sigma=0.15), F
    # the upper half of the sphere: an open mesh with one boundary loop
    keep = V[F].mean(axis=1)[:, 2] >= 0.0
    Fh = F[keep]
    used = np.unique(Fh)
    remap = -np.ones(V.shape[0], np.int64)
    remap[used] = np.arange(used.size)
    hemi = V[used].copy(), remap[Fh].astype(np.int32)
    return {"smooth": smooth, "lobed": lobed, "hemisphere": hemi}


def _cloud_of(V, F):
    """Face barycentres, unit face normals and face areas (igl::barycenter,
    igl::per_face_normals, igl::doublearea / 2)."""
    T = V[F]
    BC = T.mean(axis=1)
    cr = np.cross(T[:, 1] - T[:, 0], T[:, 2] - T[:, 0])
    dbl = np.linalg.norm(cr, axis=1)
    return BC, cr / dbl[:, None], 0.5 * dbl


def test_oracle_meshes_property():
    for name, (V, F) in _meshes().items():
        Q = V.mean(axis=0, keepdims=True)
        W_exact = O.winding_number(V, F, Q)
        W_soup = O.SoupPort(V, F, 2).eval(Q, 2.0)
        BC, N, A = _cloud_of(V, F)
        W_cloud = O.cloud_fwn(BC, N, A, Q, 2, 2.0)
        assert np.abs(W_soup - W_exact).max() < TOL_REFERENCE, name
        assert np.abs(W_cloud - W_exact).max() < TOL_REFERENCE, name
        if name != "hemisphere":
            assert abs(W_exact[0] - 1.0) < 1e-9, name   # closed, star-shaped: inside


@pytest.mark.gpu
def test_gpu_meshes_property(cuda):
    import libigl_gb300 as G
    for name, (V, F) in _meshes().items():
        c = V.mean(axis=0, keepdims=True)
        W_exact = O.winding_number(V, F, c)
        # soup, the drop-in's defaults (reference tree, order 2, accuracy 2)
        W_soup = G.fast_winding_number_soup(V, F, c)
        W_soup_ref = O.SoupPort(V, F, 2).eval(c, 2.0)
        assert np.abs(W_soup - W_exact).max() < TOL_REFERENCE, name
        assert np.abs(W_soup - W_soup_ref).max() < TOL_MIXED, name
        # cloud of face barycentres
        BC, N, A = _cloud_of(V, F)
        W64 = G.fast_winding_number_cloud_oneshot(BC, N, A, c, 2, 2.0, precision="fp64")
        Wm = G.fast_winding_number_cloud_oneshot(BC, N, A, c, 2, 2.0, precision="mixed")
        W_cloud_ref = O.cloud_fwn(BC, N, A, c, 2, 2.0)
        assert np.abs(W64 - W_cloud_ref).max() <= 1e-11, name
        assert np.abs(Wm - W64).max() <= TOL_MIXED, name
        assert np.abs(W64 - W_exact).max() < TOL_REFERENCE, name
        # exact winding number at the vertices pulled towards the centroid.
        # At these sizes the plain FP64 GPU path sums over the cap hierarchy,
        # a different split of the same sum than the oracle's triangle by
        # triangle one: on the open hemisphere the two differ by up to 4.5e-11
        # (measured), hence 1e-9 here.
        P = c + 0.8 * (V - c)
        We = G.winding_number(V, F, P, precision="fp64")
        np.testing.assert_allclose(We, O.winding_number(V, F, P), rtol=0, atol=1e-9,
                                   err_msg=name)
