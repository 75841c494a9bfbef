"""The C-ABI library builds for sm_103a, loads without a GPU, and exports every declared symbol."""

import ctypes
import os
import re

from pyseqm_gb300 import build, native

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "pyseqm_gb300.h")


def _declared():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|size_t|const char \*)\s*(seqm_\w+)\s*\(", src, re.M)))


def test_header_matches_binding_list():
    assert _declared() == sorted(native.EXPORTS)


def test_library_exports_every_declared_symbol():
    path = build.build()
    lib = ctypes.CDLL(path)
    for name in _declared():
        assert hasattr(lib, name), name
    native.load(path)
    assert b"sm_103a" in native.load().seqm_version()


def test_sp2_tc_work_size_is_host_computable():
    """The tensor-core SP2 work size is a pure host function (no GPU needed) and grows with
    the matrix total, the molecule count and the largest basis."""
    lib = native.load(build.build())
    a = lib.seqm_sp2_tc_work_bytes(100 * 100, 1, 100)
    assert a > 32 * 100 * 100
    assert lib.seqm_sp2_tc_work_bytes(2 * 100 * 100, 2, 100) > a
    assert lib.seqm_sp2_tc_work_bytes(100 * 100, 1, 200) > a


def test_batch_struct_layout_matches_header(tmp_path):
    """The ctypes seqm_batch has the header's size and field offsets (gcc on a probe that
    includes the header; no GPU): the binding and the library agree on the ABI."""
    import shutil
    import subprocess

    import pytest

    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    fields = [f[0] for f in native.SeqmBatch._fields_]
    src = tmp_path / "probe.c"
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "pyseqm_gb300.h"', "int main(void) {",
             '  printf("sizeof %zu\\n", sizeof(seqm_batch));']
    lines += [f'  printf("{f} %zu\\n", offsetof(seqm_batch, {f}));' for f in fields]
    lines += ["  return 0;", "}"]
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)], check=True)
    out = dict(line.split() for line in subprocess.run([str(exe)], check=True, capture_output=True,
                                                       text=True).stdout.splitlines())
    assert int(out["sizeof"]) == ctypes.sizeof(native.SeqmBatch)
    for f in fields:
        assert int(out[f]) == getattr(native.SeqmBatch, f).offset, f


def test_scf_state_struct_layout_matches_header(tmp_path):
    """The ctypes seqm_scf_state has the header's size and field offsets."""
    import shutil
    import subprocess

    import pytest

    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    fields = [f[0] for f in native.ScfState._fields_]
    src = tmp_path / "probe.c"
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "pyseqm_gb300.h"', "int main(void) {",
             '  printf("sizeof %zu\\n", sizeof(seqm_scf_state));']
    lines += [f'  printf("{f} %zu\\n", offsetof(seqm_scf_state, {f}));' for f in fields]
    lines += ["  return 0;", "}"]
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)], check=True)
    out = dict(line.split() for line in subprocess.run([str(exe)], check=True, capture_output=True,
                                                       text=True).stdout.splitlines())
    import ctypes as ct

    assert int(out["sizeof"]) == ct.sizeof(native.ScfState)
    for f in fields:
        assert int(out[f]) == getattr(native.ScfState, f).offset, f


def test_scf_scratch_size_matches_header(tmp_path):
    """native.scf_scratch_doubles (the fused iteration's scratch that BatchSCF allocates) agrees
    with the header's SEQM_SCF_SCRATCH_DOUBLES for a few batch shapes."""
    import shutil
    import subprocess

    import pytest

    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    shapes = [(1, 3, 3, 7), (4096, 137263, 2905604, 369032), (2, 1, 0, 1)]
    src = tmp_path / "scratch.c"
    lines = ["#include <stdio.h>", '#include "pyseqm_gb300.h"', "int main(void) {"]
    lines += [f'  printf("%zu\\n", (size_t)SEQM_SCF_SCRATCH_DOUBLES({a}, {b}, {c}, {d}));' for a, b, c, d in shapes]
    lines += ["  return 0;", "}"]
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "scratch"
    subprocess.run(["gcc", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert got == [native.scf_scratch_doubles(*s) for s in shapes]
