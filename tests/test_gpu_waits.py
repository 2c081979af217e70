"""The bounded waits of the product kernels run out without faulting or
hanging the GPU: with a short wait limit and one chunk of the producer-fed
phase 2 left out by its producer (a stage that nothing fills), the product
returns, the H-matrix's status word reports the expiry (2: a consumer gave
up, 3: the producer gave up or could not drain), a host-pointer product
fails with that status, and after the defaults are restored and the status
cleared the next product is bitwise the one before.  No counterpart in the
reference (its products run on the CPU and do not wait)."""
import numpy as np
import pytest

import htool_gb300 as H
from htool_gb300 import geometry as G

pytestmark = pytest.mark.gpu

DEFAULT_CYCLES = 4000000000


def set_waits(cycles, skip):
    H._check(H.lib.htgpu_debug_set_waits(0, cycles, skip))


def test_waits_run_out_report_and_recover():
    torch = pytest.importorskip("torch")
    n = 6000
    pts = G.sphere(n, seed=31)
    t = H.Cluster().build(n, pts)
    hm = H.HMatrix(t, t, 1e-6, 10.0).build(H.LAPLACE, pts)
    hm.set_phase2_mode(H.PHASE2_PRODUCER)
    x = G.rhs(n, 1, seed=32)
    ref = hm.mvprod_global_to_global(x)
    assert hm.device_status() == 0
    xd = torch.from_numpy(x).cuda()
    yd = torch.zeros(n, dtype=torch.float64, device="cuda")
    try:
        set_waits(2000000, 0)  # about 1 ms; chunk 0 never lands
        hm.mvprod_ptr(xd.data_ptr(), yd.data_ptr(), 1, 0, None)
        assert hm.device_status() in (2, 3)
        with pytest.raises(RuntimeError, match="device wait of the product ran out"):
            hm.mvprod_global_to_global(x)
    finally:
        set_waits(DEFAULT_CYCLES, -1)
    hm.reset_status()
    assert hm.device_status() == 0
    assert np.array_equal(hm.mvprod_global_to_global(x), ref)
    hm.mvprod_ptr(xd.data_ptr(), yd.data_ptr(), 1, 0, None)
    assert hm.device_status() == 0
    assert np.array_equal(yd.cpu().numpy(), ref)


def test_debug_waits_argument_check():
    with pytest.raises(ValueError):
        H._check(H.lib.htgpu_debug_set_waits(0, 0, -1))
