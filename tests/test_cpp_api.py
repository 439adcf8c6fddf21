"""The reference-compatible C++ API (bem2d_gb300/lib).

CPU: the reference's own driver programs (examples/, normcomps/,
numrangecomps/, resonances/) compile and link unchanged against it (needs
the reference checkout named by BEM2D_REFERENCE; skipped without); the
text output formats (WriteMatrix, WriteDensity, WriteDomain, GplotOut,
GplotOutput) byte for byte against files the reference library wrote
(tests/golden/output).
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
REF = os.environ.get("BEM2D_REFERENCE", "")


@pytest.fixture(scope="module")
def built():
    from bem2d_gb300 import _build
    _build.build_gpu()
    return _build.build_cpp()


def link(objs, out):
    subprocess.run(["g++", "-o", out] + objs + [os.path.join(LIB, "bem2d.a"), GPU_SO,
                                                "-Wl,-rpath," + os.path.dirname(GPU_SO)],
                   check=True, capture_output=True, text=True)


@pytest.mark.skipif(not REF or not os.path.isdir(os.path.join(REF, "examples")),
                    reason="BEM2D_REFERENCE does not name the reference checkout")
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


def test_output_files_match_reference(built, tmp_path):
    """tests/native/api_output.cpp writes every text format of the library;
    the reference library wrote the same program's files into
    tests/golden/output (tests/golden/make_golden.py)."""
    exe = str(tmp_path / "api_output")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + LIB,
                    os.path.join(ROOT, "tests", "native", "api_output.cpp"), "-o", exe,
                    os.path.join(LIB, "bem2d.a"), GPU_SO, "-Wl,-rpath," + os.path.dirname(GPU_SO)],
                   check=True)
    run = tmp_path / "run"
    run.mkdir()
    subprocess.run([exe], check=True, cwd=str(run))
    gold = os.path.join(ROOT, "tests", "golden", "output")
    names = sorted(os.listdir(gold))
    assert len(names) >= 12 and sorted(os.listdir(str(run))) == names
    for f in names:
        with open(os.path.join(gold, f)) as a, open(str(run / f)) as b:
            assert b.read() == a.read(), f


def _curve_speed(name):
    """|gamma'(t)| of the library curves (lib/bem2d_curvetypes.h), mpmath."""
    import mpmath as mp
    tp = 2 * mp.pi

    def kite(t):
        return mp.hypot(-tp * mp.sin(tp * t) - mp.mpf("0.65") * 2 * tp * mp.sin(2 * tp * t),
                        mp.mpf("1.5") * tp * mp.cos(tp * t))

    def trefoil(t):
        r = 1 + mp.mpf("0.3") * mp.cos(3 * tp * t)
        rp = -mp.mpf("0.3") * 3 * tp * mp.sin(3 * tp * t)
        return mp.hypot(rp, r * tp)

    def ellipse(t):
        rho = mp.mpf("1.5")
        return tp * mp.hypot(rho * mp.sin(tp * t), mp.cos(tp * t) / rho)

    def ellipsearc(t):
        th = mp.mpf("1.5") * mp.pi
        a = mp.mpf("0.3") + t * th
        return th * mp.hypot(2 * mp.sin(a), mp.cos(a))

    def invellipse(t):
        s = 1j * tp * t
        e = mp.exp(s)
        e2 = mp.exp(2 * s)
        return abs(tp * e * (1 - mp.mpf("0.2") * e2) / (1 + mp.mpf("0.2") * e2) ** 2)

    return {"circle": lambda t: tp, "kite": kite, "trefoil": trefoil, "ellipse": ellipse,
            "ellipsearc": ellipsearc, "invellipse": invellipse}[name]


def test_analytic_curve_partition_is_exact_arc_length(built, tmp_path):
    """AnalyticCurve's element end points against the exact arc-length
    partition (mpmath, 30 digits), equal and graded, for every library
    curve: within 1e-13 in the parameter.  The reference integrates
    dt/ds = 1 / |gamma'(t)| with GSL's rk2 under an absolute tolerance of
    1e-10 (lib/bem2d_shape.cpp:331-368), so its end points sit within about
    that tolerance of the same exact partition; the two libraries' elements
    differ by at most the reference's own integration error."""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 24
    exe = str(tmp_path / "api_arclength")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + LIB,
                    os.path.join(ROOT, "tests", "native", "api_arclength.cpp"), "-o", exe,
                    os.path.join(LIB, "bem2d.a"), GPU_SO, "-Wl,-rpath," + os.path.dirname(GPU_SO)],
                   check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    lines = [l.split() for l in out.splitlines() if l.strip()]
    assert len(lines) == 12
    for parts in lines:
        name, kind, ts = parts[0], parts[1], [float(v) for v in parts[2:]]
        speed = _curve_speed(name)
        length = mp.quad(speed, mp.linspace(0, 1, 9))
        # the arc-length targets of the partition, as the constructors form them
        n = len(ts) - 1
        if kind == "equal":
            targets = [i * length / n for i in range(n + 1)]
        else:
            c = max(int(np.ceil(4 * 6.0 * float(length) / 2 / np.pi)), 10)
            sig = mp.mpf("0.15")
            targets = [mp.mpf(0)] + [sig ** (3 - m) * length / c for m in range(4)]
            targets += [length / c * j for j in range(2, c)]
            targets += [length / c * (c - 1) + length / c * (1 - sig ** (m + 1)) for m in range(3)]
            targets += [length]
            assert len(targets) == n + 1, (name, len(targets), n)
        worst = 0.0
        t0, s0 = mp.mpf(0), mp.mpf(0)  # last exact point and its arc length
        for i in range(1, n):
            t = mp.mpf(ts[i])  # Newton on s(t) = target from this build's value
            for _ in range(6):
                dt = (s0 + mp.quad(speed, [t0, t]) - targets[i]) / speed(t)
                t -= dt
                if abs(dt) < mp.mpf(10) ** -20:
                    break
            worst = max(worst, abs(float(t) - ts[i]))
            t0, s0 = t, targets[i]
        assert ts[0] == 0.0 and ts[-1] == 1.0
        print(name, kind, "max |t - t_exact| = %.2e" % worst)
        assert worst < 1e-13, (name, kind, worst)
