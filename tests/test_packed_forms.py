"""The walks' packed far-field records against the reference's formulas (CPU).

The FP32 soup records (soup.cuh pack_far32) hold the order-1 and order-2
brackets of the HDK expansion (FWNFS.h:7195-7251) as a quadratic and a cubic
form in the unit direction; the cloud records (cloud.cuh pack_cloud) hold
expansion_eval (fast_winding_number.cpp:174-228) as a linear, a harmonic
quadratic and a harmonic cubic form, with three coefficients of each
harmonic form implied by the others.  A host build of the two packing
functions (tests/packed/pack_probe.cu, compiled with nvcc, run on the CPU)
packs random moments; the packed forms, evaluated here in FP64, must equal
the reference's expressions, restated below, for random directions and
distances: to FP32 rounding of the coefficients for the soup, to FP64
rounding for the cloud."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "packed", "pack_probe.cu")
OUT = os.path.join(ROOT, "tests", "packed", "_build", "pack_probe")


@pytest.fixture(scope="module")
def probe():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    subprocess.run([nvcc, "-std=c++17", "-O1", "--expt-relaxed-constexpr",
                    "-I", os.path.join(ROOT, "libigl_gb300", "csrc"),
                    "-I", os.path.join(ROOT, "include"),
                    "-gencode", "arch=compute_103a,code=sm_103a", SRC, "-o", OUT], check=True)

    def run(kind, rows):
        text = f"{kind} {len(rows)}\n" + "\n".join(" ".join(repr(float(v)) for v in r)
                                                   for r in rows) + "\n"
        r = subprocess.run([OUT], input=text, capture_output=True, text=True, check=True)
        return np.array([[float(v) for v in line.split()] for line in r.stdout.splitlines()])
    return run


def _directions(rng, n):
    u = rng.normal(size=(n, 3))
    return u / np.linalg.norm(u, axis=1, keepdims=True)


def soup_reference(m, q, r, order=2):
    """FWNFS.h:7195-7251 with q the unit direction and r = |x - P|."""
    N, Nii, (Nxy, Nyz, Nzx), Niii, perm, c2 = m[0:3], m[3:6], m[6:9], m[9:12], m[12], m[13:19]
    m1 = 1.0 / r
    m2 = m1 * m1
    qx, qy, qz = q
    om = -m2 * (q @ N)
    q2 = q * q
    om += m2 * m1 * (Nii.sum() - 3 * (q2 @ Nii + qx * qy * Nxy + qx * qz * Nzx + qy * qz * Nyz))
    t0 = np.array([c2[3] + c2[4], c2[5] + c2[0], c2[1] + c2[2]])
    t1 = np.array([qy * c2[0] + qz * c2[1], qz * c2[2] + qx * c2[3], qx * c2[4] + qy * c2[5]])
    om += m2 * m2 * (1.5 * (q @ (3 * Niii + t0))
                     - 7.5 * (q2 * q @ Niii + qx * qy * qz * perm + q2 @ t1))
    return om


def soup_packed(p, q, r):
    """omega = m2 (m1 (A(q) + m1 K(q)) - q.N), coefficients as soup.cuh lays them out."""
    bx, by, bz, bw, cx, cy, cz, cw, dx, dy, dz, dw, ex, ey, ez, ew, fx, fy, fz = p
    m1 = 1.0 / r
    m2 = m1 * m1
    qx, qy, qz = q
    x2, y2, z2, yz = qx * qx, qy * qy, qz * qz, qy * qz
    lin = qx * bx + qy * by + qz * bz
    a = qx * (bw * qx + cz * qy + cw * qz) + cx * y2 + cy * z2 + dx * yz
    k = (qx * (dy * x2 + ez * y2 + fx * z2 + fz * yz) + qy * (ex * x2 + dz * y2 + fy * z2)
         + qz * (ey * x2 + ew * y2 + dw * z2))
    return m2 * (m1 * (a + m1 * k) - lin)


def cloud_reference(ec, loc):
    """expansion_eval (fast_winding_number.cpp:174-228), loc = CM - q."""
    r = np.linalg.norm(loc)
    pi4 = 4 * np.pi
    wn = (loc @ ec[:3]) / (pi4 * r ** 3)
    sd = -3.0 / (pi4 * r ** 5) * np.outer(loc, loc) + np.eye(3) / (pi4 * r ** 3)
    wn += sd.flatten(order="F") @ ec[3:12]
    ltl = np.outer(loc, loc / (pi4 * r ** 7))
    for i in range(3):
        rcd = np.zeros((3, 3))
        for u in range(3):
            for v in range(3):
                rcd[u, v] = (loc[i] if u == v else 0) + (loc[v] if u == i else 0) + (
                    loc[u] if v == i else 0)
        td = 15.0 * loc[i] * ltl + (-3.0 / (pi4 * r ** 5)) * rcd
        wn += td.flatten(order="F") @ ec[12 + 9 * i:21 + 9 * i]
    return wn


def cloud_packed(pk, loc):
    """W = (u.N + (Q(u) + K(u)/r)/r) / r^2, Q_zz and K_xzz, K_yzz, K_zzz implied."""
    r = np.linalg.norm(loc)
    ux, uy, uz = loc / r
    x2, y2, z2, yz = ux * ux, uy * uy, uz * uz, uy * uz
    lin = ux * pk[0] + uy * pk[1] + uz * pk[2]
    qzz = -(pk[3] + pk[4])
    s = ux * (pk[3] * ux + pk[5] * uy + pk[6] * uz) + pk[4] * y2 + qzz * z2 + pk[7] * yz
    kxzz, kyzz, kzzz = -(3 * pk[8] + pk[12]), -(3 * pk[9] + pk[10]), -(pk[11] + pk[13]) / 3
    kx = pk[8] * x2 + pk[12] * y2 + kxzz * z2 + pk[14] * yz
    ky = pk[10] * x2 + pk[9] * y2 + kyzz * z2
    kz = pk[11] * x2 + pk[13] * y2 + kzzz * z2
    s += (ux * kx + uy * ky + uz * kz) / r
    return (lin + s / r) / r ** 2


def test_soup_records_equal_the_reference_far_field(probe):
    rng = np.random.default_rng(11)
    M = rng.normal(size=(300, 19)) * np.repeat([1.0, 0.3, 0.3, 0.1, 0.1, 0.1], [3, 3, 3, 3, 1, 6])
    P = probe("soup", M)
    for m, p in zip(M, P):
        for q, r in zip(_directions(rng, 4), rng.uniform(0.5, 4.0, 4)):
            ref = soup_reference(m, q, r)
            scale = np.abs(m).max() / r ** 2
            assert abs(soup_packed(p, q, r) - ref) <= 2e-6 * scale, (m, q, r)


def test_cloud_records_equal_expansion_eval(probe):
    rng = np.random.default_rng(12)
    EC = rng.normal(size=(300, 39)) * np.repeat([1.0, 0.3, 0.1], [3, 9, 27])
    PK = probe("cloud", EC)
    for ec, pk in zip(EC, PK):
        for u, r in zip(_directions(rng, 4), rng.uniform(0.5, 4.0, 4)):
            loc = u * r
            ref = cloud_reference(ec, loc)
            scale = np.abs(ec).max() / (4 * np.pi * r ** 2)
            assert abs(cloud_packed(pk, loc) - ref) <= 1e-13 * scale, (ec, loc)
