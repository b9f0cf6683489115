"""The allocation-free advem entry point (hyc_advem_noalloc).

It serves callers that cannot allocate device memory at the time they call
the advection (their device memory belongs to their own pool allocator, or
their time loop must not call cudaMalloc/cudaFree, which can synchronise the
device).  Its scratch is a fixed array inside the library, so these checks
call it twice in a row for every scheme -- the second call finds the first
call's leftovers in that array -- and compare each result bit for bit with
the oracle's advem and with hyc_advem on device pointers (the entry point
that uses the context's allocated scratch).  The file name sorts last so
that a run stopping at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import hycadv
from helpers import basin, np_case, oracle_grid, same

pytestmark = pytest.mark.gpu


def _slice_inputs(b, g, c, k, level_old, level_center, delt1):
    fld = c["temp"][level_old, k].copy()
    fldc = c["temp"][level_center, k].copy()
    u, v = c["uflx"][k].copy(), c["vflx"][k].copy()
    for a in (fld, fldc, u, v):
        g.xctilr(a, 5, 5)
    dpn = c["dp"][level_old, k]
    fd = np.zeros_like(dpn)
    fd[:-1, :-1] = ((u[:-1, 1:] - u[:-1, :-1]) + (v[1:, :-1] - v[:-1, :-1])) * delt1 * c["scp2i"][:-1, :-1]
    fco = np.maximum(dpn + fd, 0.0)
    fcn = np.maximum(dpn, 0.0)
    return [fld, fldc, u, v, fco, fcn, c["scp2"], c["scp2i"]]


def _dev(arrs, cuda):
    import torch

    return [torch.from_numpy(np.ascontiguousarray(a)).to(cuda) for a in arrs]


def _noalloc(L, b, advtyp, arrs, posdef, delt1, ip, iu, iv, stream):
    return L.hyc_advem_noalloc(b.nx, b.ny, b.nbdy, advtyp, arrs[0].data_ptr(), arrs[1].data_ptr(),
                               arrs[2].data_ptr(), arrs[3].data_ptr(), arrs[4].data_ptr(), arrs[5].data_ptr(),
                               posdef, arrs[6].data_ptr(), arrs[7].data_ptr(), delt1, ip.data_ptr(),
                               iu.data_ptr(), iv.data_ptr(), C.c_void_p(stream.cuda_stream))


@pytest.mark.parametrize("advtyp", [0, 1, 2, 4])
def test_noalloc_matches_oracle_and_advem_on_two_calls_in_a_row(cuda, advtyp):
    import torch

    b = basin(90, 70, True, seed=301)
    g = oracle_grid(b)
    delt1 = 240.0
    c = np_case(b, g, kdm=2, ntracr=0, seed=301, courant=0.8, delt1=delt1)
    sc, si = b.metrics()
    ctx = hycadv.Context.from_masks(g.masks, sc, si, kdm=1, nreg=g.nreg, nbdy=b.nbdy)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream)
    ip, iu, iv = _dev([g.masks["ip"], g.masks["iu"], g.masks["iv"]], cuda)
    L = hycadv.lib()
    calls = [(0, 1, 0, 256.0), (1, 0, 1, 0.0)]  # (layer, old level, centre level, posdef)
    for k, lo, lc, posdef in calls:
        arrs = _slice_inputs(b, g, c, k, lo, lc, delt1)
        ref = arrs[0].copy()
        g.advem(advtyp, ref, arrs[1], arrs[2], arrs[3], arrs[4], arrs[5], posdef, arrs[6], arrs[7], delt1)
        want = _dev(arrs, cuda)
        got = _dev(arrs, cuda)
        ctx.advem(advtyp, want[0], want[1], want[2], want[3], want[4], want[5], posdef, want[6], want[7], delt1)
        rc = _noalloc(L, b, advtyp, got, posdef, delt1, ip, iu, iv, stream)
        assert rc == 0, hycadv._err()
        torch.cuda.synchronize()
        out = got[0].cpu().numpy()
        assert same(out, ref), f"advtyp {advtyp} layer {k}: differs from the oracle's advem"
        assert same(out, want[0].cpu().numpy())
        assert not np.array_equal(out, arrs[0])
    ctx.close()


def test_noalloc_rejects_oversized_slice_and_wide_halo(cuda):
    import torch

    L = hycadv.lib()
    dummy = torch.zeros(8, dtype=torch.float64, device=cuda)
    p = dummy.data_ptr()
    idm = jdm = 1500  # (1500+12)^2 cells > 2^21
    rc = L.hyc_advem_noalloc(idm, jdm, 6, 2, p, p, p, p, p, p, 0.0, p, p, 1.0, p, p, p, None)
    assert rc == -1
    assert "static scratch" in hycadv._err()
    rc = L.hyc_advem_noalloc(10, 10, 1 << 30, 2, p, p, p, p, p, p, 0.0, p, p, 1.0, p, p, p, None)
    assert rc == -1
    assert "nbdy" in hycadv._err()


def test_noalloc_rejects_inconsistent_masks(cuda):
    """An iu that is not ip(i)*ip(i-1) is reported (HYC_ERR_MASK), as
    hyc_adv_init reports it; the next call with the bigrid masks is exact."""
    import torch

    b = basin(60, 50, False, seed=302)
    g = oracle_grid(b)
    delt1 = 600.0
    c = np_case(b, g, kdm=1, ntracr=0, seed=302, courant=0.6, delt1=delt1)
    arrs = _slice_inputs(b, g, c, 0, 1, 0, delt1)
    stream = torch.cuda.current_stream()
    L = hycadv.lib()
    bad_iu = g.masks["iu"].copy()
    jj, ii = np.argwhere(g.masks["iu"] != 0)[len(np.argwhere(g.masks["iu"] != 0)) // 2]
    bad_iu[jj, ii] = 0
    ip, iu, iv, iub = _dev([g.masks["ip"], g.masks["iu"], g.masks["iv"], bad_iu], cuda)
    got = _dev(arrs, cuda)
    rc = _noalloc(L, b, 2, got, 0.0, delt1, ip, iub, iv, stream)
    assert rc == -4  # HYC_ERR_MASK
    assert "inconsistent" in hycadv._err()
    got = _dev(arrs, cuda)
    assert _noalloc(L, b, 2, got, 0.0, delt1, ip, iu, iv, stream) == 0
    ref = arrs[0].copy()
    g.advem(2, ref, arrs[1], arrs[2], arrs[3], arrs[4], arrs[5], 0.0, arrs[6], arrs[7], delt1)
    torch.cuda.synchronize()
    assert same(got[0].cpu().numpy(), ref)
