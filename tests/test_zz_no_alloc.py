"""The allocation-free force entry point (cuibm_cv_force_noalloc).

Some callers cannot allocate GPU memory at the point where they need the body
force: a host framework or coupling code whose memory pool has reserved the
device (a cudaMalloc there fails or fragments the pool), or a time-stepping
loop that cannot take the device-wide synchronisation cudaMalloc and cudaFree
imply.  cuibm_cv_force_noalloc serves them: the caller passes device
arrays it already owns, and the kernel's scratch is a fixed array inside the
library.  This file is collected last so that a failure here cannot hide
another test's; it must pass alone in a fresh process and after the suite.
"""
import ctypes

import numpy as np
import pytest

cb = pytest.importorskip("cuibm_gb300")
torch = pytest.importorskip("torch")
from cuibm_gb300 import cases  # noqa: E402

pytestmark = pytest.mark.gpu

RTOL = 1e-12  # the two paths sum the same terms in a different block order


def _device_copy(s, name, dtype):
    n = s.field_size(name)
    t = torch.empty(n, dtype=dtype, device="cuda")
    s.get_into(name, t.data_ptr(), t.numel() * t.element_size(), on_device=True)
    return t


def test_noalloc_force_matches_context_force(tmp_path):
    f = cases.cylinder(str(tmp_path / "c"), h=0.05, ratio=1.1, extent=3.0, core=0.6, points=48, nu=0.025,
                       dt=0.01, nt=20)
    L = cb.library()
    with cb.NavierStokesSolver(f) as s:
        s.set_option("write_output", 0)
        s.initialise()
        s.stepTime(5)
        s.run("force")  # the existing entry point: context kernel, context scratch
        fx, fy = s.forces()
        i = s.info
        u = _device_copy(s, "u", torch.float64)
        uold = _device_copy(s, "uold", torch.float64)
        p = _device_copy(s, "p", torch.float64)
        tags = _device_copy(s, "ghost_tags_uv", torch.int32)
        dx = _device_copy(s, "dx", torch.float64)
        dy = _device_copy(s, "dy", torch.float64)
        torch.cuda.synchronize()
        for call in range(2):  # two calls in a row share (and must reset) the scratch
            out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
            st = L.cuibm_cv_force_noalloc(u.data_ptr(), uold.data_ptr(), p.data_ptr(), tags.data_ptr(),
                                          dx.data_ptr(), dy.data_ptr(), i.nx, i.ny, i.bb_start_i, i.bb_start_j,
                                          i.bb_ncx, i.bb_ncy, i.nu, i.dt, out.data_ptr(), None)
            assert st == cb.OK, L.cuibm_case_error()
            torch.cuda.synchronize()
            gx, gy = out.cpu().tolist()
            assert abs(gx - fx) <= RTOL * max(1.0, abs(fx)), (call, gx, fx)
            assert abs(gy - fy) <= RTOL * max(1.0, abs(fy)), (call, gy, fy)
        assert abs(fx) > 1e-6  # a real drag, not an empty sum


def test_noalloc_force_rejects_oversized_box():
    L = cb.library()
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check fails first
    st = L.cuibm_cv_force_noalloc(dummy, dummy, dummy, dummy, dummy, dummy, 4000, 4000, 10, 10, 600, 600, 0.01, 0.01,
                                  dummy, None)
    assert st == cb.ERR_BAD_INPUT
    assert b"exceeds the limit" in L.cuibm_case_error()


@pytest.mark.parametrize("box", [(10, 10, 20, 89), (10, 10, 89, 20)])
def test_noalloc_force_rejects_box_at_grid_edge(box):
    """A box whose north edge reaches row ny - 1 (v has rows 0..ny-2) or whose east edge
    reaches column nx - 1 (u has columns 0..nx-2) would read past the arrays."""
    L = cb.library()
    dummy = ctypes.c_void_p(16)  # never dereferenced: the range check fails first
    st = L.cuibm_cv_force_noalloc(dummy, dummy, dummy, dummy, dummy, dummy, 100, 100, *box, 0.01, 0.01, dummy, None)
    assert st == cb.ERR_BAD_INPUT
    assert b"out of range" in L.cuibm_case_error()
