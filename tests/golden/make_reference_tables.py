"""Writes tests/golden/reference_tables.npz: the literal test inputs that the
reference's GPU tests hold for the P2G / G2P path, read as text from its
source (the reference is Rust and cannot run here).

  many_positions        rust/crates/gpu/src/test_util.rs:112-631  (the 8^3
                        lattice the scatter / collect / step tests use at
                        grid_node_size 0.5)
  specific_positions,   rust/crates/gpu/src/test_util.rs:678-2729 (positions
  specific_bits         and collider bits of the register_contributors,
                        prepare_grid and step tests)
  simple_gradients      rust/crates/gpu/src/test_util.rs:633-676
                        (test_position_gradients_simple, row-major literals,
                        stored column-major like nalgebra)
  lame_parameters       rust/crates/util/src/elastic.rs:679-689
                        ([E, nu] pairs of test_lame_parameters)
  inviscid_parameters   rust/crates/util/src/elastic.rs:691-693
                        ([bulk modulus, exponent] of test_inviscid_parameters)

Run from the repository root with the reference checked out:
    python tests/golden/make_reference_tables.py /root/reference
"""

from __future__ import annotations

import re
import sys
from pathlib import Path

import numpy as np

FLOAT = r"-?\d+(?:\.\d*)?(?:[eE][-+]?\d+)?"


def _function_body(text: str, name: str) -> str:
    start = text.index(f"pub fn {name}(")
    brace = text.index("{", start)
    depth = 0
    for i in range(brace, len(text)):
        if text[i] == "{":
            depth += 1
        elif text[i] == "}":
            depth -= 1
            if depth == 0:
                return text[brace:i + 1]
    raise ValueError(name)


def _vec3s(body: str) -> np.ndarray:
    rows = re.findall(rf"Vector3::new\(\s*({FLOAT}),\s*({FLOAT}),\s*({FLOAT})\s*\)", body)
    return np.array([[float(a), float(b), float(c)] for a, b, c in rows], np.float32)


def main(reference: Path) -> None:
    util = (reference / "rust/crates/gpu/src/test_util.rs").read_text()
    elastic = (reference / "rust/crates/util/src/elastic.rs").read_text()

    many = _vec3s(_function_body(util, "many_positions"))
    spec_body = _function_body(util, "specific_positions_and_collider_bits")
    spec = _vec3s(spec_body)
    bits = np.array([int(b) for b in re.findall(r"collider_bits:\s*(\d+)", spec_body)], np.uint32)
    assert len(spec) == len(bits) > 0

    simple = []
    for block in re.findall(r"from_row_slice\(&\[(.*?)\]\)", _function_body(util, "test_position_gradients_simple"),
                            re.S):
        vals = [float(v) for v in re.findall(FLOAT, block.replace("//", " "))]
        assert len(vals) == 9
        row_major = np.array(vals, np.float32).reshape(3, 3)
        simple.append(row_major.T.reshape(9))  # column-major, like nalgebra's storage
    simple.insert(0, np.eye(3, dtype=np.float32).reshape(9))  # Matrix3::identity()

    lame_body = _function_body(elastic, "test_lame_parameters")
    lame = np.array([[float(a), float(b)] for a, b in re.findall(rf"\[({FLOAT}),\s*({FLOAT})\]", lame_body)],
                    np.float64)
    inv_body = _function_body(elastic, "test_inviscid_parameters")
    inviscid = np.array([[float(a), int(b)] for a, b in re.findall(rf"\(({FLOAT}),\s*(\d+)\)", inv_body)],
                        np.float64)

    out = Path(__file__).resolve().parent / "reference_tables.npz"
    np.savez_compressed(out, many_positions=many, specific_positions=spec, specific_bits=bits,
                        simple_gradients=np.array(simple, np.float32), lame_parameters=lame,
                        inviscid_parameters=inviscid)
    print(f"{out}: {len(many)} lattice positions, {len(spec)} specific positions, {len(simple)} gradients, "
          f"{len(lame)} Lame and {len(inviscid)} inviscid parameter sets")


if __name__ == "__main__":
    main(Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference"))
