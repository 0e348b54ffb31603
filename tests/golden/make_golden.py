"""Generates tests/golden/oracle_small_mixed.npz: inputs and outputs of the
fp64 CPU oracle (the reference MPM substep restated, oracle/) on a small
seeded multi-material scene.  These vectors are produced by our restatement,
not by the reference (which cannot be built here); they guard the oracle
against regressions and give the GPU path a fixed target.

Run from the repository root:  python tests/golden/make_golden.py
"""

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from squishy_volumes_gb300 import scenes  # noqa: E402

SUBSTEPS = 3
FIELDS = ["flags", "positions", "position_gradients", "velocities", "velocity_gradients", "mass", "initial_volume",
          "mu", "lambda_", "sand_alpha", "exponent", "bulk_modulus", "viscosity_dynamic", "viscosity_bulk", "model",
          "hardening", "crit_compression", "crit_stretch", "plastic_j"]
OUT_FIELDS = ["flags", "positions", "position_gradients", "velocities", "velocity_gradients", "elastic_energies",
              "plastic_j"]


def build_scene():
    return scenes.small_mixed(n_per_material=27, seed=11, dx=0.05)


def main():
    s = build_scene()
    p = s.io_state.particles
    o = oracle.OracleState(p, s.consts, s.extras, fp64=True, threads=1)
    assert o.step(SUBSTEPS, s.dt, s.gravity) == 0
    out = o.download()
    data = {f"in_{k}": getattr(p, k) for k in FIELDS}
    data.update({f"out_{k}": getattr(out, k) for k in OUT_FIELDS})
    data["dt"] = np.float32(s.dt)
    data["gravity"] = np.asarray(s.gravity, np.float32)
    data["substeps"] = np.int32(SUBSTEPS)
    data["grid_node_size"] = np.float32(s.consts.grid_node_size)
    data["domain_min"] = np.asarray(s.consts.domain_min, np.float32)
    data["domain_max"] = np.asarray(s.consts.domain_max, np.float32)
    np.savez_compressed(Path(__file__).with_name("oracle_small_mixed.npz"), **data)
    print("wrote", p.n, "particles")


if __name__ == "__main__":
    main()
