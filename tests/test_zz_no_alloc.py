"""sp_bs4_dot_f64_noalloc -- the BS4 dot for callers that cannot allocate device
memory (their memory belongs to another allocator or a fixed pool, or they cannot
afford cudaMalloc's device-wide synchronisation), so they cannot hand over the
partial-sum buffer that sp_bs4_1_f64 needs.  Its partials live in a static array
of the library.

Checked through the C ABI against the oracle's restatement of the reference's
bs4_1/bs4_2 (the same partition and tree, with the CUDA mode's fma) and against
the two-stage entry points (sp_bs4_1_f64 + sp_reduce_finish_f64 with a
caller-allocated partial buffer): the results must agree bit for bit -- the
tolerance every order-exact reduction test here uses.  Two calls in a row, the
second with fewer blocks than the first for every block size, show that the
shared array carries nothing from one call into the next.  This file is collected
last so that a run stopping at the first failure has run every other test."""
import pytest
import torch

from streamparanumal_gb300 import capi

pytestmark = pytest.mark.gpu


def two_stage(bs, nb, n, a, b, stream):
    tmp = torch.zeros(bs, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    capi.call("sp_bs4_1_f64", bs, nb, n, a.data_ptr(), b.data_ptr(), tmp.data_ptr(), stream)
    capi.call("sp_reduce_finish_f64", bs, nb, tmp.data_ptr(), out.data_ptr(), stream)
    return out


def nblocks(n, bs):
    return max(1, min((n + bs - 1) // bs, bs))


@pytest.mark.parametrize("bs", [256, 1024])
def test_noalloc_dot_matches_two_stage_dot_on_consecutive_calls(cuda, orc, bs):
    stream = torch.cuda.current_stream().cuda_stream
    # two calls in a row; the second has fewer blocks (20,001 < 256 * 256 entries)
    for n, seed in ((1_000_003, 5), (20_001, 9)):
        ha, hb = orc.uniform(n, seed), orc.uniform(n, seed + 1)
        a, b = torch.from_numpy(ha).cuda(), torch.from_numpy(hb).cuda()
        nb = nblocks(n, bs)
        got = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        capi.call("sp_bs4_dot_f64_noalloc", bs, nb, n, a.data_ptr(), b.data_ptr(),
                  got.data_ptr(), stream)
        want = two_stage(bs, nb, n, a, b, stream)
        torch.cuda.synchronize()
        _, ref = orc.bs4(ha, hb, bs=bs, nblocks=nb, fmad=1)
        assert got.item() == ref
        assert got.item() == want.item()


def test_noalloc_dot_rejects_more_blocks_than_its_array_holds(cuda):
    st = capi.status("sp_bs4_dot_f64_noalloc", 1024, 1025, 10, None, None, None, None)
    assert st == capi.SP_ERR_SIZE
    assert "capacity" in capi.last_error()
