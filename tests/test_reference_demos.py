"""The reference's own demo programs that use only the GPU API compile
unchanged against include/HLanc.hpp and link against libhlanc_gb300
(tests/cpp/build_reference_demos.sh; skipped where the reference sources are
absent).  matrix_convertor needs no GPU: its binary CSR output must be
byte-identical to this library's own writer on the same input."""
import os
import subprocess

import pytest

from conftest import ROOT, GOLDEN


@pytest.fixture(scope="module")
def demos(tmp_path_factory):
    from hlanc_gb300 import build
    build.build()
    out = tmp_path_factory.mktemp("refdemos")
    r = subprocess.run(["sh", os.path.join(ROOT, "tests", "cpp", "build_reference_demos.sh"), str(out)],
                       capture_output=True, text=True)
    if r.returncode == 3:
        pytest.skip("reference demo sources absent")
    assert r.returncode == 0, r.stderr[-2000:]
    return out


def test_demos_build(demos):
    for f in ("matrix_convertor", "verify_eigs", "HLanc_solver_gpu"):
        assert os.path.exists(demos / f)


READERS = sorted(f for f in os.listdir(os.path.join(GOLDEN, "readers")) if f.endswith((".mtx", ".pp")))


@pytest.mark.parametrize("name", READERS)
def test_matrix_convertor_output_matches_library_writer(demos, tmp_path, name):
    import hlanc_gb300 as H
    fmt = "mm" if name.endswith(".mtx") else "pp"
    src = os.path.join(GOLDEN, "readers", name)
    out = tmp_path / "demo.bin"
    subprocess.run([str(demos / "matrix_convertor"), fmt, src, str(out)], check=True, capture_output=True)
    mine = tmp_path / "mine.bin"
    H.dcsr_matrix_t(fmt, src).save_bin(str(mine))
    assert out.read_bytes() == mine.read_bytes()
