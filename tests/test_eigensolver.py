"""The closed-form 3x3 symmetric eigensolver of the learned closure
(sym_eig3 in squishy_volumes_gb300/csrc/sv_eig.cuh, host-compiled here by
nvcc) against numpy's eigh, on deformation gradients of the kinds the
substep produces: near identity down to 1e-13 perturbations (where the
shifted rows' cross products would underflow without scaling), strong
random deformations, double roots and rotations."""

import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "squishy_volumes_gb300" / "csrc"

DRIVER = r"""
#include <cstdio>
#include "sv_eig.cuh"
int main() {
    float a[6], lam[3], V[9];
    while (scanf("%f %f %f %f %f %f", &a[0], &a[1], &a[2], &a[3], &a[4], &a[5]) == 6) {
        sv::sym_eig3(a, lam, V);
        printf("%.9g %.9g %.9g", lam[0], lam[1], lam[2]);
        for (int k = 0; k < 9; ++k) printf(" %.9g", V[k]);
        printf("\n");
    }
    return 0;
}
"""


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    d = tmp_path_factory.mktemp("eig")
    (d / "drv.cu").write_text(DRIVER)
    subprocess.run([nvcc, "-std=c++17", "-I", str(CSRC), "-I", str(ROOT / "include"), "-o", str(d / "drv"),
                    str(d / "drv.cu")], check=True, capture_output=True)
    return d / "drv"


def _cases(seed=0, n=600):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        kind = k % 6
        if kind == 0:
            F = np.eye(3) + 1e-3 * rng.normal(size=(3, 3))
        elif kind == 1:
            F = np.eye(3) + 10.0 ** rng.uniform(-13, -7) * rng.normal(size=(3, 3))
        elif kind == 2:
            F = rng.normal(size=(3, 3))
        elif kind == 3:
            Q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
            F = Q @ np.diag([1.0, 1.0, 0.9])  # double root of F^T F
        elif kind == 4:
            Q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
            F = Q * (1 + 1e-6 * rng.normal(size=3))  # near rotation
        else:
            F = np.eye(3) + 0.05 * rng.normal(size=(3, 3))
        out.append((kind, F.astype(np.float32)))
    return out


def test_sym_eig3_matches_eigh(driver):
    cases = _cases()
    lines = []
    for _, F in cases:
        f = F.astype(np.float32)
        c = [f[:, 0] @ f[:, 0], f[:, 0] @ f[:, 1], f[:, 0] @ f[:, 2], f[:, 1] @ f[:, 1], f[:, 1] @ f[:, 2],
             f[:, 2] @ f[:, 2]]
        lines.append(" ".join(f"{np.float32(x):.9g}" for x in c))
    res = subprocess.run([str(driver)], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
    rows = res.stdout.strip().split("\n")
    assert len(rows) == len(cases)
    for (kind, F), row in zip(cases, rows):
        v = np.array([float(x) for x in row.split()])
        assert np.isfinite(v).all(), kind
        lam, V = v[:3], v[3:].reshape(3, 3).T  # columns are eigenvectors
        C = F.astype(np.float64).T @ F.astype(np.float64)
        ref = np.sort(np.linalg.eigvalsh(C))[::-1]
        assert np.all(np.diff(lam) <= 1e-6 * ref[0]), (kind, lam)  # descending
        assert np.max(np.abs(lam - ref)) <= 2e-6 * ref[0], (kind, lam, ref)
        assert np.max(np.abs(V.T @ V - np.eye(3))) <= 3e-6, kind
        assert np.max(np.abs(C @ V - V * lam)) <= 3e-6 * ref[0], kind
        # the SVD it implies reconstructs F
        S = np.sqrt(lam)
        U = (F.astype(np.float64) @ V) / S
        assert np.max(np.abs(U @ np.diag(S) @ V.T - F)) <= 3e-6 * max(1.0, S[0]), kind
