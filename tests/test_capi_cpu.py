"""The C-ABI library builds for sm_103a, loads, and exports every entry point
include/bem2d_gpu.h declares.  No GPU compute happens here."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "bem2d_gpu.h")


def declared():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"\b(bem2d_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from bem2d_gb300 import _build
    _build.build_gpu()
    from bem2d_gb300 import capi
    return capi.load()


def test_exports_every_declared_symbol(lib):
    names = declared()
    assert len(names) >= 12
    for n in names:
        assert hasattr(lib, n), n
    from bem2d_gb300 import capi
    assert sorted(capi.EXPORTS) == names


def test_binding_constants_match_header():
    """The ctypes binding's kernel, functional and precision codes are the
    header's #defines (no library load needed)."""
    from bem2d_gb300 import capi
    src = open(HEADER).read()
    defs = {m.group(1): int(m.group(2))
            for m in re.finditer(r"#define\s+(BEM2D_\w+)\s+(-?\d+)", src)}
    for table, prefix in ((capi.KERNEL, "BEM2D_KERNEL_"), (capi.FUN, "BEM2D_FUN_"),
                          (capi.PREC, "BEM2D_PREC_")):
        names = {k: v for k, v in defs.items() if k.startswith(prefix)}
        assert sorted(table.values()) == sorted(names.values()), (prefix, table, names)
        for key, code in table.items():
            assert defs[prefix + key.upper()] == code, (prefix, key)


def test_noalloc_layout_fits_at_the_limit(lib):
    """The allocation-free solve's work buffers for n = BEM2D_NOALLOC_MAX_N
    fit its static device array (host-side arithmetic only)."""
    from bem2d_gb300 import capi
    fits, need, cap = capi.noalloc_scratch_fits()
    assert fits, (need, cap)
    assert 16 * capi.NOALLOC_MAX_N ** 2 < need <= cap


def test_gauss_host_rule_matches_oracle(lib):
    from bem2d_gb300 import capi, _build
    from oracle import oracle as O
    _build.build_oracle(with_reference=False)
    for n in (1, 2, 5, 7, 16, 30):
        x, w = capi.gauss(n)
        xo, wo = O.gauss(n)
        assert np.abs(x - xo).max() < 1e-15 and np.abs(w - wo).max() < 1e-15


def test_context_without_gpu_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = lib.bem2d_ctx_create(0, ctypes.byref(h))
    assert rc != 0 and not h.value


def test_sm103a_code_in_library(lib):
    """The library carries sm_103a device code (checked through cuobjdump's
    listing of embedded ELF architectures, not by disassembly)."""
    import shutil
    import subprocess
    from bem2d_gb300 import capi
    tool = shutil.which("cuobjdump") or "/usr/local/cuda/bin/cuobjdump"
    if not os.path.exists(tool):
        pytest.skip("cuobjdump not available")
    out = subprocess.run([tool, "--list-elf", capi.LIB_PATH], capture_output=True, text=True).stdout
    assert "sm_103a" in out


def test_leading_dimension_of_torch_views():
    """The binding's leading dimension for column-major torch views (the
    solve and assembly entry points take it from the tensor): a transposed
    contiguous tensor, a padded buffer's transposed view, and row-major
    storage read as the transpose; numpy arrays are taken as n."""
    torch = pytest.importorskip("torch")
    from bem2d_gb300 import capi
    n = 5
    a = torch.zeros((n, n), dtype=torch.complex128)
    assert capi._ld(a.T.contiguous().T, n) == n
    buf = torch.zeros((n, n + 7), dtype=torch.complex128)
    assert capi._ld(buf.t(), n) == n + 7
    assert capi._ld(a, n) == n
    assert capi._ld(np.zeros((n, n), order="F"), n) == n
