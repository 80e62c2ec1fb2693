"""The C-ABI boundary without a GPU: the library loads, exports every entry
point include/caustics_gb300.h declares, its host-only entry points work, its
argument checks reject bad calls before any launch, and the Python mirrors
refuse to run without a CUDA device (no CPU fallback)."""
import ctypes
import os
import re

import numpy as np
import pytest
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "caustics_gb300.h")


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    return sorted(set(re.findall(r"^\s*[A-Za-z_][\w\s\*]*?\b((?:cgb|gpu)_\w+)\s*\(", text, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    from caustics_gb300 import _lib as L
    if not os.path.exists(L.LIB_PATH):
        from caustics_gb300 import build
        build.build()
    return L.lib()


def test_header_declares_the_entry_points():
    names = declared_functions()
    for n in ("cgb_ea_solve", "gpu_ehrlich_aberth", "cgb_ea_roots_jvp", "cgb_ea_roots_vjp", "cgb_mag_point_source",
              "cgb_mag_extended_source", "cgb_mag_extended_source_grad", "cgb_mag", "cgb_mag_lc_batched",
              "cgb_mag_lc_batched_vjp", "cgb_mag_lc_batched_workspace_bytes"):
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_host_entry_points(lib):
    from caustics_gb300 import _lib as L
    assert lib.cgb_abi_version() == 6
    for n in (2, 7, 50, 100):
        x = np.zeros(n)
        w = np.zeros(n)
        assert lib.cgb_gauss_legendre(n, x.ctypes.data_as(ctypes.c_void_p), w.ctypes.data_as(ctypes.c_void_p)) == 0
        xr, wr = np.polynomial.legendre.leggauss(n)
        assert np.allclose(np.sort(x), xr, atol=1e-14) and np.allclose(w[np.argsort(x)], wr, atol=1e-14)
    assert lib.cgb_mag_lc_batched_workspace_bytes(1000) >= 16 + 8 * 1000
    assert lib.cgb_mag_lc_batched_vjp_workspace_bytes(1000) == 16 + 80 * 1000
    assert L.CGB_ERR_UNSUPPORTED == 3


def test_argument_checks_before_any_launch(lib):
    from caustics_gb300 import _lib as L
    assert lib.cgb_ea_solve(None, None, None, 0, 7, 100, 0, None, None) == L.CGB_ERR_UNSUPPORTED
    assert b"degree" in lib.cgb_last_error()
    assert lib.cgb_ea_solve(None, None, None, -1, 5, 100, 0, None, None) == L.CGB_ERR_INVALID
    assert lib.cgb_ea_solve(None, None, None, 4, 5, 100, 0, None, None) == L.CGB_ERR_INVALID  # null buffers
    assert lib.cgb_ea_roots_jvp(None, None, None, None, 0, 0, None) == L.CGB_ERR_INVALID
    bad = L.LensParams(2, -1.0, 0.1, 0, 0, 0)
    assert lib.cgb_mag_point_source(None, None, None, None, 0, bad, 100, 0, None, None) == L.CGB_ERR_INVALID
    assert lib.cgb_ea_solve(None, None, None, 0, 5, 100, 0, None, None) == L.CGB_OK  # empty batch: no launch
    # batched workspace: 16 + 16 n bytes asked for; below the queue alone (16 + 8 n) the call is refused
    n = 100
    assert lib.cgb_mag_lc_batched_workspace_bytes(n) == 16 + 16 * n
    buf = np.zeros(64)
    ptr = buf.ctypes.data_as(ctypes.c_void_p)
    opts = L.EsOptions(200, 1, 0.5, 100, 2500, 1, 0, 1, 1, 0, 0.0)
    rc = lib.cgb_mag_lc_batched(ptr, ptr, ptr, 1, n, ptr, ptr, None, ctypes.byref(opts), ptr, 16 + 8 * n - 1, None)
    assert rc == L.CGB_ERR_INVALID and b"workspace" in lib.cgb_last_error()


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the behaviour without a CUDA device")
def test_no_cpu_fallback(lib):
    import caustics_gb300 as C
    from caustics_gb300 import _lib as L
    with pytest.raises(L.CausticsError):
        C.mag_point_source(np.array([0.1 + 0.1j]), s=0.9, q=0.1)
    with pytest.raises(L.CausticsError):
        C.mag_extended_source(0.1 + 0.1j, 1e-2, s=0.9, q=0.1)


def test_ctypes_structs_match_the_header(tmp_path):
    """The Python mirror's ctypes structures have the size and field offsets of
    the C structs in include/caustics_gb300.h (a C program compiled against the
    header reports them)."""
    import shutil
    import subprocess
    from caustics_gb300 import _lib as L
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {"cgb_lens_params": L.LensParams, "cgb_es_options": L.EsOptions, "cgb_curve_params": L.CurveParams}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "caustics_gb300.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    inc = os.path.join(ROOT, "include")
    cuda_inc = "/usr/local/cuda/include"
    subprocess.run([cc, "-std=c11", "-I", inc, "-I", cuda_inc, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
