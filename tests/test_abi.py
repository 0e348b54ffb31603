"""The C ABI (CPU only, no compute calls): the built library loads and
exports every function include/*.h declares, and the ctypes mirrors used by
the host side match the C struct layouts (checked against gcc)."""

import ctypes as ct
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_functions():
    names = set()
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b(sv_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ["sv_create", "sv_step", "sv_download", "sv_download_grid", "sv_destroy", "sv_last_error_string"]:
        assert required in names


def test_library_exports_every_declared_symbol(cuda_lib):
    missing = [n for n in declared_functions() if not hasattr(cuda_lib, n)]
    assert not missing, missing


def test_struct_layouts_match_c(tmp_path):
    from squishy_volumes_gb300._abi import SvConsts, SvParticles, SvStats

    src = tmp_path / "layout.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "squishy_volumes_cuda.h"\n'
        "int main(void) {\n"
        '  printf("%zu %zu %zu\\n", sizeof(sv_consts), sizeof(sv_particles), sizeof(sv_stats));\n'
        '  printf("%zu %zu %zu\\n", offsetof(sv_consts, block_capacity), offsetof(sv_consts, sort_interval),'
        " offsetof(sv_particles, plastic_j));\n"
        "  return 0;\n}\n"
    )
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("gcc unavailable: " + r.stderr)
    sizes, offsets = subprocess.run([str(exe)], capture_output=True, text=True).stdout.split("\n")[:2]
    assert [int(x) for x in sizes.split()] == [ct.sizeof(SvConsts), ct.sizeof(SvParticles), ct.sizeof(SvStats)]
    assert [int(x) for x in offsets.split()] == [SvConsts.block_capacity.offset, SvConsts.sort_interval.offset,
                                                 SvParticles.plastic_j.offset]


def test_frame_input_layout_matches_c_and_the_oracle(tmp_path):
    from oracle.oracle import OFrameInput
    from squishy_volumes_gb300._abi import SvFrameInput

    fields = [f[0] for f in SvFrameInput._fields_]
    assert fields == [f[0] for f in OFrameInput._fields_]
    src = tmp_path / "frame.c"
    lines = "".join(f'  printf("%zu ", offsetof(sv_frame_input, {f}));\n' for f in fields)
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "squishy_volumes_cuda.h"\n'
                   "int main(void) {\n" + lines + '  printf("%zu\\n", sizeof(sv_frame_input));\n  return 0;\n}\n')
    exe = tmp_path / "frame"
    r = subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("gcc unavailable: " + r.stderr)
    vals = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    assert vals[:-1] == [getattr(SvFrameInput, f).offset for f in fields]
    assert vals[-1] == ct.sizeof(SvFrameInput) == ct.sizeof(OFrameInput)


def test_frame_layout_matches_c(tmp_path):
    from squishy_volumes_gb300._abi import SvFrame

    fields = [f[0] for f in SvFrame._fields_]
    c_names = ["lambda" if f == "lambda_" else f for f in fields]
    src = tmp_path / "sv_frame.c"
    lines = "".join(f'  printf("%zu ", offsetof(sv_frame, {f}));\n' for f in c_names)
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "squishy_volumes_cuda.h"\n'
                   "int main(void) {\n" + lines + '  printf("%zu\\n", sizeof(sv_frame));\n  return 0;\n}\n')
    exe = tmp_path / "sv_frame"
    r = subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("gcc unavailable: " + r.stderr)
    vals = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    assert vals[:-1] == [getattr(SvFrame, f).offset for f in fields]
    assert vals[-1] == ct.sizeof(SvFrame)


def test_oracle_is_not_linked_by_the_product():
    """The product library must not depend on the CPU oracle."""
    from squishy_volumes_gb300 import build

    lib = build.library_path()
    r = subprocess.run(["ldd", str(lib)], capture_output=True, text=True)
    assert "sv_oracle" not in r.stdout
    for src in (ROOT / "squishy_volumes_gb300").rglob("*"):
        if src.suffix in (".py", ".cu", ".cuh", ".h", ".cpp"):
            text = src.read_text()
            assert "import oracle" not in text and "sv_oracle" not in text, src
