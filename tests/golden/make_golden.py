"""Generate the committed golden fixtures from the reference library itself.

Builds oracle/_ref/ref_dump (the reference's lib/ compiled in place with the
shims in oracle/shim, see oracle/Makefile), runs it on every case in
cases.py, and stores the outputs as tests/golden/<case>.npz.

Small cases keep full matrices.  Larger ones keep size-independent probes:
A @ v and A^H @ w for seeded vectors, the diagonal, 4096 seeded entries, the
right-hand side, the solution and the norm / condition number.

The text output formats: oracle/_ref/ref_output (tests/native/api_output.cpp
linked to the reference library) writes its files into tests/golden/output.

Run from the repository root, with the reference checkout named:
    BEM2D_REFERENCE=<checkout> python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from golden.cases import CASES, QUAD  # noqa: E402

REF_DUMP = os.path.join(ROOT, "oracle", "_ref", "ref_dump")
REF_OUTPUT = os.path.join(ROOT, "oracle", "_ref", "ref_output")


def output_files():
    """The reference library's text output files (api_output.cpp) into
    tests/golden/output, replacing what is there."""
    out = os.path.join(ROOT, "tests", "golden", "output")
    os.makedirs(out, exist_ok=True)
    for f in os.listdir(out):
        os.remove(os.path.join(out, f))
    subprocess.run([REF_OUTPUT], check=True, cwd=out)
    return sorted(os.listdir(out))


def probes(A, seed):
    rng = np.random.default_rng(seed)
    n = A.shape[0]
    v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    w = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    ii = rng.integers(0, n, 4096)
    jj = rng.integers(0, n, 4096)
    return dict(probe_v=v, probe_w=w, Av=A @ v, AHw=A.conj().T @ w,
                diag=np.diag(A).copy(), sample_i=ii, sample_j=jj,
                sample=A[ii, jj], fro=np.linalg.norm(A))


def read_c(path, shape):
    return np.fromfile(path, dtype=np.complex128).reshape(shape, order="F")


def run_case(name, spec):
    g = spec["geom"]()
    n = g.n_unknowns
    k, eta, d = spec["k"], spec["eta"], spec["direction"]
    kim = spec.get("kim", 0.0)
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        lines = g.to_refspec(QUAD)
        if spec.get("scattering", True):
            lines.append("op scattering %.17g %.17g %.17g %.17g %.17g %s/sys"
                         % (k, kim, d[0], d[1], eta, tmp))
        lines.append("op ident %s/ident.bin" % tmp)
        for kn in spec.get("kernels", ()):
            lines.append("op kernel %s %.17g %.17g %.17g %s/k_%s.bin"
                         % (kn, k, kim, eta, tmp, kn))
        if spec.get("numrange"):
            lines.append("op numrange %.17g %.17g %.17g %d %s/numrange.txt"
                         % (k, kim, eta, spec["numrange"], tmp))
        if spec.get("singvals"):
            lines.append("op singvals %.17g %.17g %.17g %s/singvals.bin" % (k, kim, eta, tmp))
        if spec.get("evalsol"):
            pts = spec["evalsol"]
            lines.append("op evalsol %.17g %.17g %.17g %.17g %.17g %s/evalsol.bin %s"
                         % (k, kim, d[0], d[1], eta, tmp,
                            " ".join("%.17g %.17g" % p for p in pts)))
        with open(os.path.join(tmp, "case.txt"), "w") as f:
            f.write("\n".join(lines) + "\n")
        subprocess.run([REF_DUMP, os.path.join(tmp, "case.txt")], check=True,
                       stdout=subprocess.DEVNULL)
        out["ident_diag"] = np.diag(read_c(tmp + "/ident.bin", (n, n))).copy()
        if spec.get("scattering", True):
            A = read_c(tmp + "/sys_A.bin", (n, n))
            out["rhs"] = np.fromfile(tmp + "/sys_rhs.bin", dtype=np.complex128)
            out["x"] = np.fromfile(tmp + "/sys_x.bin", dtype=np.complex128)
            out["normcond"] = np.fromfile(tmp + "/sys_normcond.bin", dtype=np.float64)
            if spec["full"]:
                out["A"] = A
            else:
                out.update(probes(A, 1234))
        for kn in spec.get("kernels", ()):
            out["K_" + kn] = read_c("%s/k_%s.bin" % (tmp, kn), (n, n))
        if spec.get("evalsol"):
            out["evalsol_points"] = np.array(spec["evalsol"], dtype=np.float64)
            out["evalsol"] = np.fromfile(tmp + "/evalsol.bin", dtype=np.complex128)
        if spec.get("numrange"):
            pts = np.loadtxt(tmp + "/numrange.txt")
            out["numrange"] = pts[:, 0] + 1j * pts[:, 1]
        if spec.get("singvals"):
            out["singvals"] = np.fromfile(tmp + "/singvals.bin", dtype=np.float64)
    meta = dict(name=name, n=n, k=k, eta=eta, direction=list(d), quad=list(QUAD))
    if kim:
        meta["kim"] = kim
    out["meta"] = np.array(json.dumps(meta))
    return out


def hankel_fixture():
    """BesselH0 / BesselH1 of a complex argument through the reference's own
    routines (lib/bem2d_mathroutines.cpp:44-75) and the binary128 zbesh shim,
    at seeded points of the complex evaluator's domain; checked here against
    scipy.special.hankel1 (AMOS zbesh itself)."""
    import scipy.special as sp
    rng = np.random.default_rng(2024)
    r = 10 ** rng.uniform(-5, np.log10(300), 600)
    a = rng.uniform(-np.pi / 3, np.pi / 2, 600)
    z = r * np.exp(1j * a)
    z = z[z.imag < 60]
    with tempfile.TemporaryDirectory() as tmp:
        lines = ["quad 3 5 0.15", "seg 0 0 1 0 0 -1 -1", "basis poly 0",
                 "op hankel %s/h.bin %s" % (tmp, " ".join("%.17g %.17g" % (x.real, x.imag)
                                                          for x in z))]
        with open(os.path.join(tmp, "case.txt"), "w") as f:
            f.write("\n".join(lines) + "\n")
        subprocess.run([REF_DUMP, os.path.join(tmp, "case.txt")], check=True,
                       stdout=subprocess.DEVNULL)
        h = np.fromfile(tmp + "/h.bin", dtype=np.complex128).reshape(-1, 2)
    for nu in (0, 1):
        e = np.abs(h[:, nu] - sp.hankel1(nu, z)) / np.abs(sp.hankel1(nu, z)) / (1 + np.abs(z) / 50)
        assert e.max() < 4e-15, ("zbesh shim vs scipy AMOS", nu, e.max())
    return dict(z=z, h0=h[:, 0].copy(), h1=h[:, 1].copy())


def main():
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    ref = os.environ.get("BEM2D_REFERENCE", "")
    if not ref:
        raise SystemExit("set BEM2D_REFERENCE to the reference checkout")
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "-j8", "ref", "REF=" + ref],
                   check=True, stdout=subprocess.DEVNULL)
    names = sys.argv[1:] or (list(CASES) + ["hankel_ck", "output"])
    for name in names:
        if name == "output":
            print("output files:", " ".join(output_files()))
            continue
        if name == "hankel_ck":
            path = os.path.join(ROOT, "tests", "golden", "hankel_ck.npz")
            np.savez_compressed(path, **hankel_fixture())
            print("%-16s %7.1f KB" % (name, os.path.getsize(path) / 1024))
            continue
        res = run_case(name, CASES[name])
        path = os.path.join(ROOT, "tests", "golden", name + ".npz")
        np.savez_compressed(path, **res)
        print("%-16s n=%-5d %7.1f KB" % (name, json.loads(str(res["meta"]))["n"],
                                          os.path.getsize(path) / 1024))


if __name__ == "__main__":
    main()
