"""The C ABI without a GPU: libvtg.so builds for sm_103a, loads, exports every function include/*.h declares, and its
host-only entry points answer. No kernel runs here."""
import ctypes as C
import glob
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        # the native entry points (vtg_*) and the reference-signature ones (*_cuda, vtg_compat.h)
        for m in re.finditer(r"\b(vtg_[a-z0-9_]+|[a-z0-9_]+_cuda)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_entry_points():
    names = declared_functions()
    assert "vtg_build" in names and "vtg_cells" in names and "vtg_points" in names
    assert {"img_u8_to_q6_cuda", "img_reduce_cuda", "lk_track_cuda", "lk_flowback_cuda", "lk_tile_bytes_cuda",
            "still_vectors_cuda", "tk_correlate_cuda"} <= set(names)


def test_library_exports_every_declared_symbol(vtg_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", vtg_lib.LIB_PATH], capture_output=True, text=True, check=True)
    exported = {line.split()[-1] for line in out.stdout.splitlines() if " T " in line}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, "declared but not exported: %s" % missing
    lib = vtg_lib.lib()
    for n in declared_functions():
        assert hasattr(lib, n)


def test_host_only_entry_points(vtg_lib):
    lib = vtg_lib.lib()
    assert lib.vtg_strerror(vtg_lib.EBUDGET).decode().startswith("over")
    cfg = vtg_lib.config(1920, 1080, levels=4, cell_w=16, cell_h=8)
    b = lib.vtg_tracker_bytes(C.byref(cfg))
    # two sets of F32 planes (pitch 1920, 960, 480, 256) plus staging and 16,200 cells
    assert b > 2 * 4 * (1920 * 1080 + 960 * 540 + 480 * 270 + 256 * 135) and b < 40_000_000
    for bad in (dict(levels=0), dict(levels=7), dict(patch_w=31), dict(patch_h=33), dict(flow_level=4),
                dict(cell_w=0), dict(max_iter=0)):
        kw = dict(width=1920, height=1080, levels=4, cell_w=16, cell_h=8)
        kw.update(bad)
        assert lib.vtg_tracker_bytes(C.byref(vtg_lib.config(**kw))) == 0, bad


def test_contrast_gain_matches_oracle(vtg_lib):
    """vtg_contrast_gain (the host copy of the function the build options' kernel runs) against the oracle's integer
    restatement of tk_build's x87 gain and offset, for every byte min / max pair (x 64) and some wider ranges."""
    import numpy as np

    import oracle as O

    lib = vtg_lib.lib()
    go = (C.c_float * 2)()
    pairs = [(64 * a, 64 * b) for a in range(256) for b in range(a, 256)]
    pairs += [(0, 16777215), (5, 16777215), (123456, 123457), (3, 7), (16000000, 16700001)]
    for lo, hi in pairs:
        assert lib.vtg_contrast_gain(lo, hi, go) == 0
        want = O.contrast_gain(lo, hi)
        assert np.array(go[:], np.float32).view(np.uint32).tolist() == want.view(np.uint32).tolist(), (lo, hi)
    assert lib.vtg_contrast_gain(5, 4, go) == vtg_lib.EINVAL
    assert lib.vtg_contrast_gain(-1, 4, go) == vtg_lib.EINVAL
    assert lib.vtg_contrast_gain(0, 1 << 24, go) == vtg_lib.EINVAL


def _build_c_caller(vtg_lib, out_dir):
    """tests/c/track_pair.c compiled as C11 and linked against libvtg.so, as the reference's host code would be."""
    exe = os.path.join(str(out_dir), "track_pair")
    lib_dir = os.path.dirname(vtg_lib.LIB_PATH)
    subprocess.run(["cc", "-std=c11", "-O2", "-Wall", "-Wextra", "-Werror", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c", "track_pair.c"), "-o", exe, "-L" + lib_dir, "-lvtg",
                    "-Wl,-rpath," + lib_dir, "-lm"], check=True, capture_output=True, text=True)
    return exe


def test_c_caller_builds_and_links(vtg_lib, tmp_path):
    """The public headers are C11 (the reference's language), and a C program links against libvtg.so."""
    exe = _build_c_caller(vtg_lib, tmp_path)
    assert os.path.exists(exe)


def test_context_without_gpu_is_refused(vtg_lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert vtg_lib.lib().vtg_ctx_create(0, 0, C.byref(h)) == vtg_lib.ENODEV


def test_no_fallback_without_library(tmp_path, monkeypatch, vtg_lib):
    """The binding refuses to run without the compiled library: no CPU fallback exists."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("vtg_copy", os.path.join(os.path.dirname(vtg_lib.__file__), "vtg.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    monkeypatch.setattr(mod, "LIB_PATH", str(tmp_path / "missing.so"))
    with pytest.raises(RuntimeError):
        mod.lib()
