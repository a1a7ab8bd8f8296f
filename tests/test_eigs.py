"""The eigenpair text format of the reference demo (written by
demo/HLanc_solver_gpu.cu:57-66, read by demo/verify_eigs.cu:8-44): nev, n,
the nev eigenvalues, then n rows of nev vector entries, all "%23.15lE".
CPU tests: the writer's bytes equal the reference format rendered here, the
reader takes that format back exactly, errors are status codes, and the
header-only C++ API (HLanc::write_eigs / HLanc::eigs_t) agrees."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

INC = os.path.join(ROOT, "include")


@pytest.fixture(scope="module")
def H():
    import hlanc_gb300 as H
    from hlanc_gb300 import build
    build.build()
    return H


def _reference_text(vals, vecs):
    nev, n = len(vals), vecs.shape[0]
    out = [f"{nev}\n{n}\n"] + ["%23.15E\n" % v for v in vals]
    for r in range(n):
        out.append(" ".join("%23.15E" % vecs[r, c] for c in range(nev)) + "\n")
    return "".join(out)


def _sample(n=37, nev=5, seed=11):
    rng = np.random.default_rng(seed)
    vals = np.sort(rng.standard_normal(nev)) * np.array([1e-300, 1.0, -3.5, 1e200, 7e-17])[:nev]
    vecs = rng.standard_normal((n, nev)) * np.logspace(-12, 12, n)[:, None]
    vecs[3, 1] = 0.0
    vecs[4, 2] = -0.0
    return vals, np.asfortranarray(vecs)


def test_writer_bytes_match_reference_format(H, tmp_path):
    vals, vecs = _sample()
    p = tmp_path / "eigs.txt"
    H.write_eigs(str(p), vals, vecs)
    assert p.read_text() == _reference_text(vals, vecs)


def test_reader_takes_reference_format(H, tmp_path):
    vals, vecs = _sample(n=21, nev=3, seed=4)
    p = tmp_path / "ref.txt"
    p.write_text(_reference_text(vals, vecs))
    got_v, got_x = H.read_eigs(str(p))
    toks = p.read_text().split()
    want_v = np.array([float(t) for t in toks[2:2 + 3]])
    want_x = np.array([float(t) for t in toks[2 + 3:]]).reshape(21, 3)
    assert np.array_equal(got_v, want_v)
    assert np.array_equal(got_x, want_x)
    assert np.abs(got_x - vecs).max() <= 1e-14 * np.abs(vecs).max()


def test_errors_are_status_codes(H, tmp_path):
    with pytest.raises(H.HLancError) as e:
        H.read_eigs(str(tmp_path / "missing.txt"))
    assert e.value.status == 6
    p = tmp_path / "short.txt"
    p.write_text("2\n3\n1.0\n")
    with pytest.raises(H.HLancError) as e:
        H.read_eigs(str(p))
    assert e.value.status == 6


def test_cpp_header_api(H, tmp_path):
    src = tmp_path / "eigs.cpp"
    src.write_text(r'''
#include <cstdio>
#include "HLanc.hpp"
int main(int argc, char **argv) {
    double vals[2] = {-1.25, 3.0e-7};
    double vecs[6] = {1, 2, 3, 4.5, -5, 6e10};
    if (HLanc::write_eigs(argv[1], 2, 3, vals, vecs, 3)) return 3;
    HLanc::eigs_t e;
    if (e.load(argv[1])) return 4;
    bool ok = e.nev == 2 && e.n == 3;
    for (int i = 0; i < 2; ++i) ok = ok && e.value[i] == vals[i];
    for (int i = 0; i < 6; ++i) ok = ok && e.vector[i] == vecs[i];
    printf("%d\n", ok ? 1 : 0);
    return 0;
}
''')
    exe = tmp_path / "eigs"
    libdir = os.path.dirname(H.LIB_PATH)
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-I", INC, str(src), "-o", str(exe), "-L", libdir,
                           "-lhlanc_gb300", f"-Wl,-rpath,{libdir}"])
    out = subprocess.check_output([str(exe), str(tmp_path / "e.txt")]).decode().split()
    assert out == ["1"]
