"""Failure detection on the GPU without a fault: a bounded device wait that
nothing completes gives up, reports through the error flag, and leaves the
device and the library usable (the streaming kernels' failure path; the
reference has no recovery path, its errors stop the model with xcstop)."""
import time

import pytest

import hycadv
from helpers import basin, np_case, oracle_grid, same
from test_gpu_parity import bind_all, gpu_steps, make_ctx, oracle_steps, torchify

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_device_stays_usable(cuda):
    import torch

    assert hycadv.selftest_wait(arrive=True) == 0
    t0 = time.perf_counter()
    assert hycadv.selftest_wait(arrive=False) == 1  # nothing completes the barrier
    waited = time.perf_counter() - t0
    assert 1.5 < waited < 30.0, waited  # the wait's limit is 2 s of device time
    assert hycadv.selftest_wait(arrive=True) == 0
    # the library still advects correctly on the same device
    b = basin(40, 30, False, seed=17)
    g = oracle_grid(b)
    c = np_case(b, g, kdm=2, ntracr=0, seed=17, courant=0.5, delt1=1800.0)
    c["delt1"] = 1800.0
    t = torchify(c, cuda)
    ctx = make_ctx(b, g, 2)
    bind_all(ctx, t)
    gpu_steps(ctx, c, range(1, 3), 2)
    oracle_steps(g, c, range(1, 3), 2)
    torch.cuda.synchronize()
    for k in ("temp", "saln"):
        assert same(t[k].cpu().numpy(), c[k]), k
    ctx.close()


def test_selftest_argument_errors(cuda):
    with pytest.raises(hycadv.HycError) as e:
        hycadv._check(hycadv.lib().hyc_selftest_wait(0, 1, None))
    assert e.value.code == -1
    with pytest.raises(hycadv.HycError) as e:
        hycadv.selftest_wait(True, device=1 << 20)
    assert e.value.code == -5
