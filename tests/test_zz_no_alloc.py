"""vtg_search_run_noalloc: the appearance search for callers that cannot allocate device memory at the moment they search
(a real-time loop that cannot absorb a cudaMalloc, a host runtime that owns every byte of device memory). Its scratch is
one fixed device array that every call shares, so this test checks, through the C ABI, that calls in a row each give
the existing vtg_search_run's answer (the map's corners and the found corner exactly, scores within 1e-6):
  - a 640 x 480 Q6 plane, then a 320 x 240 8-bit plane with another template, so nothing left from the first call can
    pass for a result of the second;
  - then 640 x 480 again with another seed, window and step: its integral-image rows and map cells past the 320 x 240
    call's reach still hold the first call's values, so a call that read scratch it had not rewritten would differ.
It also checks that sizes past the limits are refused. The same calls run once more in a child process of their own,
where the library is loaded fresh and the first call on the device makes the address lookup."""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle as O
import vtg_synth as S

pytestmark = pytest.mark.gpu


def _noalloc(vtg_lib):
    L = vtg_lib.lib()
    L.vtg_search_run_noalloc.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int,
                                         C.c_float, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.vtg_search_run_noalloc.restype = C.c_int
    return L.vtg_search_run_noalloc


def _case(w, h, seed, tw, th, tx, ty, plane_type):
    frame = S.noise_frame(w, h, seed=seed)
    plane = O.pyramid(frame, 1)[0] if plane_type == 1 else frame
    app, norm = O.cut_template(plane.astype(np.float32), tx, ty, tw, th)
    return plane, app, norm


def test_noalloc_matches_search_run(vtg_lib, ctx):
    import torch

    run = _noalloc(vtg_lib)
    cases = [((640, 480, 31, 32, 21, 300, 200, 1), (1, 640, 1, 480, 1)),  # a Q6 plane, the reference's template size
             ((320, 240, 57, 64, 48, 40, 150, 0), (20, 300, 10, 230, 2)),  # an 8-bit plane, another template
             ((640, 480, 83, 48, 32, 500, 380, 1), (7, 629, 3, 470, 4))]  # 640 x 480 again: reads past the last call's
    for (w, h, seed, tw, th, tx, ty, ptype), (x0, x1, y0, y1, step) in cases:
        plane, app, norm = _case(w, h, seed, tw, th, tx, ty, ptype)
        dplane = torch.from_numpy(np.ascontiguousarray(plane)).cuda()
        dapp = torch.from_numpy(np.ascontiguousarray(app)).cuda()
        cells = ((min(x1, w - tw - 2) - max(x0, 1)) // 16 + 1) * ((min(y1, h - th - 2) - max(y0, 1)) // 16 + 1)
        dfound = torch.zeros(8, dtype=torch.int32, device="cuda")  # struct vtg_found, 32 bytes
        dmv = torch.zeros(cells, dtype=torch.float32, device="cuda")
        dmx = torch.zeros(cells, dtype=torch.int32, device="cuda")
        dmy = torch.zeros(cells, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        rc = run(dplane.data_ptr(), w, h, w, ptype, dapp.data_ptr(), tw, th, norm, x0, x1, y0, y1, step,
                 dfound.data_ptr(), dmv.data_ptr(), dmx.data_ptr(), dmy.data_ptr(), None)
        assert rc == vtg_lib.OK
        torch.cuda.synchronize()
        got = vtg_lib.Found.from_buffer_copy(dfound.cpu().numpy().tobytes()).as_dict()

        s = vtg_lib.Search(ctx, w, h, 64, 64)
        s.template(app, norm)
        ref, rv, rx, ry = s.run(dplane.data_ptr(), w, h, w, ptype, x0, x1, y0, y1, step, want_map=True)
        s.close()
        assert got["cells"] == ref["cells"] == cells
        assert (got["hx"], got["hy"], got["ntop"]) == (ref["hx"], ref["hy"], ref["ntop"])
        for k in ("ncc", "second", "ox", "oy"):
            assert abs(got[k] - ref[k]) <= 1e-6, k
        assert np.array_equal(dmx.cpu().numpy(), rx) and np.array_equal(dmy.cpu().numpy(), ry)
        assert np.abs(dmv.cpu().numpy() - rv).max() <= 1e-6


def test_noalloc_refuses_past_its_limits(vtg_lib):
    import torch

    run = _noalloc(vtg_lib)
    big = torch.zeros((720, 1280), dtype=torch.uint8, device="cuda")
    app = torch.zeros((21, 32), dtype=torch.float32, device="cuda")
    found = torch.zeros(8, dtype=torch.int32, device="cuda")
    # a 1280 x 720 plane is past the scratch's size; a 96-wide template past its template limit
    assert run(big.data_ptr(), 1280, 720, 1280, 0, app.data_ptr(), 32, 21, 1.0, 1, 1280, 1, 720, 1, found.data_ptr(),
               None, None, None, None) == vtg_lib.EINVAL
    assert run(big.data_ptr(), 320, 240, 1280, 0, app.data_ptr(), 96, 21, 1.0, 1, 320, 1, 240, 1, found.data_ptr(),
               None, None, None, None) == vtg_lib.EINVAL


@pytest.mark.skipif(os.environ.get("VTG_NOALLOC_CHILD") == "1", reason="already the child process")
def test_noalloc_in_a_fresh_process():
    """The calls above in a process that has never loaded the library: its first call on the device looks the scratch
    array's address up."""
    here = os.path.dirname(os.path.abspath(__file__))
    env = dict(os.environ, VTG_NOALLOC_CHILD="1")
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-p", "no:cacheprovider", "-m", "gpu",
                        os.path.join(here, "test_zz_no_alloc.py") + "::test_noalloc_matches_search_run"],
                       cwd=os.path.dirname(here), env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
