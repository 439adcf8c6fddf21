"""The reference-compatible C++ API (bem2d_gb300/lib).

CPU: the reference's own driver programs (examples/, normcomps/,
numrangecomps/, resonances/) compile and link unchanged against it (needs
the reference checkout; skipped without).
GPU: a program written against the API reproduces the reference's disk
results (tests/golden/disk160.npz)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "bem2d_gb300", "lib")
GPU_SO = os.path.join(ROOT, "bem2d_gb300", "libbem2d_gpu.so")
REF = os.environ.get("BEM2D_REFERENCE", "/root/reference")


@pytest.fixture(scope="module")
def built():
    from bem2d_gb300 import _build
    _build.build_gpu()
    return _build.build_cpp()


def link(objs, out):
    subprocess.run(["g++", "-o", out] + objs + [os.path.join(LIB, "bem2d.a"), GPU_SO,
                                                "-Wl,-rpath," + os.path.dirname(GPU_SO)],
                   check=True, capture_output=True, text=True)


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "examples")),
                    reason="reference checkout not present")
@pytest.mark.parametrize("sub", ["examples", "normcomps", "numrangecomps", "resonances"])
def test_reference_drivers_compile_and_link_unchanged(built, tmp_path, sub):
    """Each driver #includes "../lib/bem2d.h": a sibling lib/ directory that is
    this build's API makes them compile as they are."""
    os.symlink(LIB, tmp_path / "lib")
    (tmp_path / sub).mkdir()
    names = sorted(f for f in os.listdir(os.path.join(REF, sub)) if f.endswith(".cpp"))
    assert names
    for f in names:
        shutil.copy(os.path.join(REF, sub, f), tmp_path / sub / f)
        src = str(tmp_path / sub / f)
        obj = src[:-4] + ".o"
        r = subprocess.run(["g++", "-std=gnu++17", "-O1", "-c", src, "-o", obj],
                           capture_output=True, text=True)
        assert r.returncode == 0, (f, r.stderr[-2000:])
        link([obj], src[:-4])


@pytest.mark.gpu
def test_api_program_matches_reference(built, tmp_path):
    exe = str(tmp_path / "api_disk")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + LIB,
                    os.path.join(ROOT, "tests", "native", "api_disk.cpp"), "-o", exe,
                    os.path.join(LIB, "bem2d.a"), GPU_SO, "-Wl,-rpath," + os.path.dirname(GPU_SO)],
                   check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    vals = [l.split() for l in out.splitlines() if l and l[0] in "-0123456789"]
    z = np.load(os.path.join(ROOT, "tests", "golden", "disk160.npz"))
    norm, cond = map(float, vals[0])
    assert abs(norm - z["normcond"][0]) < 1e-11 * norm
    assert abs(cond - z["normcond"][1]) < 1e-9 * cond
    n2, c2 = map(float, vals[1])
    assert abs(n2 - norm) < 1e-11 * norm and abs(c2 - cond) < 1e-9 * cond
    u = np.array([complex(float(a), float(b)) for a, b in vals[2:6]])
    assert np.linalg.norm(u - z["evalsol"]) < 1e-11 * np.linalg.norm(z["evalsol"])
    a00 = complex(float(vals[6][0]), float(vals[6][1]))
    assert abs(a00 - z["A"][0, 0]) < 1e-13 * abs(z["A"][0, 0])


def test_api_complex_hankel_host(built, tmp_path):
    """BesselH0 / BesselH1 of a complex argument and SingleLayer at a complex
    wavenumber, evaluated on the host by the C++ API, against the reference's
    own values (tests/golden/hankel_ck.npz)."""
    exe = str(tmp_path / "api_hankel")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + LIB,
                    os.path.join(ROOT, "tests", "native", "api_hankel.cpp"), "-o", exe,
                    os.path.join(LIB, "bem2d.a"), GPU_SO, "-Wl,-rpath," + os.path.dirname(GPU_SO)],
                   check=True)
    z = np.load(os.path.join(ROOT, "tests", "golden", "hankel_ck.npz"))
    pts = z["z"]
    inp = "".join("%.17g %.17g\n" % (p.real, p.imag) for p in pts)
    out = subprocess.run([exe], input=inp, check=True, capture_output=True, text=True).stdout
    v = np.array([[float(t) for t in l.split()] for l in out.splitlines()])
    h0 = v[:, 0] + 1j * v[:, 1]
    h1 = v[:, 2] + 1j * v[:, 3]
    sl = v[:, 4] + 1j * v[:, 5]
    scale = 1 + np.abs(pts) / 50
    assert (np.abs(h0 - z["h0"]) / np.abs(z["h0"]) / scale).max() < 4e-15
    assert (np.abs(h1 - z["h1"]) / np.abs(z["h1"]) / scale).max() < 4e-15
    assert (np.abs(sl - 0.25j * z["h0"]) / np.abs(z["h0"]) / scale).max() < 4e-15
