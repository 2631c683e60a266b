"""BS0-BS5 CUDA kernels against the oracle (GPU).

Copy and axpy are bit-exact; the order-exact reductions are bit-exact with the
oracle's restatement of the reference's two-stage tree under CUDA-mode
contraction (fmad); the single-launch reductions are within a stated bound of a
double-double reference; FP32-storage results are within 1e-6 relative of the
FP64 oracle."""
import numpy as np
import pytest
import torch

from streamparanumal_gb300 import kernels as K

pytestmark = pytest.mark.gpu

SIZES = [0, 1, 2, 3, 31, 255, 256, 257, 1023, 1024, 1025, 4095, 65537, 1 << 20, (1 << 20) + 3]


def dev(x):
    return torch.from_numpy(x).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("offset", [0, 1])
def test_bs1_copy_bit_exact(cuda, orc, n, offset):
    a = orc.uniform(n + offset, 11 + n)
    da = dev(a)[offset:]
    db = torch.full((n + offset,), 7.0, dtype=torch.float64, device="cuda")[offset:]
    K.bs1(n, da, db)
    np.testing.assert_array_equal(host(db), a[offset:])
    # f32
    a32 = a.astype(np.float32)
    da32 = dev(a32)[offset:]
    db32 = torch.zeros(n + offset, dtype=torch.float32, device="cuda")[offset:]
    K.bs1(n, da32, db32)
    np.testing.assert_array_equal(host(db32), a32[offset:])


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("ab", [(1.0, 1.0), (0.37, -1.9), (-0.731, 0.5)])
def test_bs2_axpy_bit_exact(cuda, orc, n, ab):
    alpha, beta = ab
    x = orc.uniform(n, 100 + n)
    y = orc.uniform(n, 200 + n)
    dy = dev(y)
    K.bs2(n, alpha, dev(x), beta, dy)
    np.testing.assert_array_equal(host(dy), orc.bs2(alpha, x, beta, y, fmad=1))
    x32, y32 = x.astype(np.float32), y.astype(np.float32)
    dy32 = dev(y32)
    K.bs2(n, alpha, dev(x32), beta, dy32)
    np.testing.assert_array_equal(host(dy32), orc.bs2(alpha, x32, beta, y32, fmad=1))


def test_bs2_misaligned_vectors(cuda, orc):
    n = 1001
    x = orc.uniform(n + 1, 5)
    y = orc.uniform(n + 1, 6)
    dx, dy = dev(x), dev(y)
    K.bs2(n, 0.25, dx[1:], -3.0, dy[:n])  # x is 8-byte aligned only
    np.testing.assert_array_equal(host(dy)[:n], orc.bs2(0.25, x[1:].copy(), -3.0, y[:n].copy()))


@pytest.mark.parametrize("n", [1, 5, 256, 257, 65536, 65537, 300000, 1 << 21])
@pytest.mark.parametrize("bs", [256, 1024])
def test_bs3_order_exact(cuda, orc, n, bs):
    a = orc.uniform(n, 300 + n)
    if n > 300:  # magnitudes over a wide range, and exact zeros, in some chains
        a[::97] *= 2.0 ** -300
        a[::89] = 0.0
    nb = K.nblocks_for(n, bs)
    tmp = torch.zeros(bs, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    K.bs3_1(nb, n, dev(a), tmp, block_size=bs)
    K.bs3_2(nb, tmp, out, block_size=bs)
    part, res = orc.bs3(a, bs=bs, nblocks=nb, fmad=1)
    np.testing.assert_array_equal(host(tmp)[:nb], part)
    assert host(out)[0] == res


@pytest.mark.parametrize("n", [1, 7, 257, 65537, 1 << 20, (1 << 21) + 5])
@pytest.mark.parametrize("bs", [256, 512])
def test_bs4_order_exact(cuda, orc, n, bs):
    a = orc.uniform(n, 400 + n)
    b = orc.uniform(n, 500 + n)
    nb = K.nblocks_for(n, bs)
    tmp = torch.zeros(bs, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    K.bs4_1(nb, n, dev(a), dev(b), tmp, block_size=bs)
    K.bs4_2(nb, tmp, out, block_size=bs)
    part, res = orc.bs4(a, b, bs=bs, nblocks=nb, fmad=1)
    np.testing.assert_array_equal(host(tmp)[:nb], part)
    assert host(out)[0] == res
    # and the dot is within 1e-14 relative... of the exact value only when no
    # cancellation; the fixed order is what makes it reproducible
    exact = orc.dot_dd(a, b)
    assert abs(res - exact) <= 1e-12 * max(1.0, np.abs(a * b).sum())


@pytest.mark.parametrize("n", [1, 1023, 1024, 1025, 1 << 20, (1 << 21) + 9])
@pytest.mark.parametrize("bs", [1024, 256])
def test_bs5_order_exact(cuda, orc, n, bs):
    Ap = orc.uniform(n, 600 + n)
    r = orc.uniform(n, 700 + n)
    alpha = -0.6180339887
    nb = K.nblocks_for(n, bs)
    dr = dev(r)
    tmp = torch.zeros(bs, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    K.bs5_1(nb, n, dev(Ap), alpha, dr, tmp, block_size=bs)
    K.bs5_2(nb, tmp, out, block_size=bs)
    r_ref, part, res = orc.bs5(Ap, alpha, r, bs=bs, nblocks=nb, fmad=1)
    np.testing.assert_array_equal(host(dr), r_ref)
    np.testing.assert_array_equal(host(tmp)[:nb], part)
    assert host(out)[0] == res


def test_reference_driver_nblock_rule():
    # Nblock = min(ceil(N/bs), bs) (BS/BS3/src/bs3Run.cpp:80-81)
    assert K.nblocks_for(1, 256) == 1
    assert K.nblocks_for(257, 256) == 2
    assert K.nblocks_for(1 << 28, 256) == 256
    assert K.nblocks_for(1 << 28, 1024) == 1024


@pytest.mark.parametrize("n", [0, 1, 3, 1000, 65537, 1 << 22])
def test_fast_reductions_fp64(cuda, orc, n):
    a = orc.uniform(n, 800 + n)
    b = orc.uniform(n, 900 + n)
    sc = K.ReduceScratch()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    K.dot(dev(a), dev(b), out, sc)
    exact = orc.dot_dd(a, b)
    # fixed-grid FP64 dot (short lane chains, then a tree): within 1e-14 of the
    # cancellation-free scale sum|ab|; relative to the result itself no order but
    # the exact one can promise that when the terms cancel
    assert abs(host(out)[0] - exact) <= 1e-14 * float(np.abs(a * b).sum())
    K.norm2(dev(a), out, sc)
    exact = orc.dot_dd(a, a)
    # integer-pipe sum of squares: within 4 ulps of the double-double sum
    assert abs(host(out)[0] - exact) <= 4 * np.spacing(exact)
    # scratch is left zeroed: a second call gives the same bits
    first = host(out)[0]
    K.norm2(dev(a), out, sc)
    assert host(out)[0] == first


def norm_inputs(orc, n, kind):
    a = orc.uniform(n, 1300 + n)
    rng = np.random.default_rng(n)
    if kind == "wide":  # magnitudes 2^-600 .. 2^200, every binade spacing
        a *= np.exp2(rng.integers(-600, 200, n).astype(np.float64))
    elif kind == "zeros":  # mostly exact zeros (and -0.0)
        a[rng.random(n) < 0.9] = 0.0
        a[::7] = -0.0
    elif kind == "tails":  # a few large values, the rest 2^-20 .. 2^-40 below them
        a *= np.exp2(-rng.integers(20, 40, n).astype(np.float64))
        a[::1009] = rng.uniform(-1, 1, a[::1009].size) * 2.0 ** 10
    elif kind == "subnormal":
        a *= 2.0 ** -1060
        a[::2] *= 2.0 ** 500
    return a


@pytest.mark.parametrize("n", [1, 2, 1 << 10, (1 << 16) + 3, 1 << 20, (1 << 22) + 1])
@pytest.mark.parametrize("kind", ["uniform", "wide", "zeros", "tails", "subnormal"])
def test_bs3_fast_norm(cuda, orc, n, kind):
    """The drivers' default BS3 (integer-pipe stage 1 + the reference's stage 2):
    within 4 ulps of the double-double sum, and within 1e-14 relative of the
    reference's order-exact result, for uniform, wide-magnitude (2^-600..2^200),
    zero-heavy, heavy-tailed and subnormal inputs."""
    a = norm_inputs(orc, n, kind)
    nb = K.nblocks_for(n, 256)
    tmp = torch.full((256,), float("nan"), dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    K.bs3_1_fast(nb, n, dev(a), tmp, K.ReduceScratch())
    K.bs3_2(nb, tmp, out)
    got = host(out)[0]
    assert np.all(host(tmp)[1:nb] == 0.0)
    exact = orc.dot_dd(a, a)
    assert abs(got - exact) <= 4 * np.spacing(exact)
    _, ref = orc.bs3(a, bs=256, nblocks=nb, fmad=1)
    assert abs(got - ref) <= 1e-14 * ref


@pytest.mark.parametrize("n", [1, 2, 1 << 10, (1 << 16) + 3, (1 << 22) + 1])
@pytest.mark.parametrize("kind", ["uniform", "wide", "zeros", "subnormal"])
@pytest.mark.parametrize("bs", [1024, 256])
def test_bs5_fast_update(cuda, orc, n, kind, bs):
    """The drivers' default BS5 (r update as the reference stores it, r.r on the
    integer pipe, then the reference's stage 2): r bit for bit as the order-exact
    bs5_1 (CUDA fma), r.r within 4 ulps of the double-double sum of the stored r and
    within 1e-14 relative of the reference's order-exact result."""
    Ap = norm_inputs(orc, n, kind)
    r0 = orc.uniform(n, 77 + n)
    alpha = 0.37
    nb = K.nblocks_for(n, bs)
    r = dev(r0)
    tmp = torch.full((bs,), float("nan"), dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    K.bs5_1_fast(nb, n, dev(Ap), alpha, r, tmp, K.ReduceScratch(), block_size=bs)
    K.reduce_finish(nb, tmp, out, block_size=bs)
    want_r, _, ref = orc.bs5(Ap, alpha, r0, bs=bs, nblocks=nb, fmad=1)
    np.testing.assert_array_equal(host(r), want_r)
    assert np.all(host(tmp)[1:nb] == 0.0)
    got = host(out)[0]
    exact = orc.dot_dd(want_r, want_r)
    assert abs(got - exact) <= 4 * np.spacing(exact)
    assert abs(got - ref) <= 1e-14 * ref


def test_bs3_fast_norm_special_values(cuda, orc):
    sc = K.ReduceScratch()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    for vals, want in (([1.0, np.inf, 2.0], np.inf), ([1.0, np.nan, 3.0], np.nan),
                       ([np.inf, -np.inf], np.inf), ([1e200, 1e200], np.inf),
                       ([0.0, -0.0, 0.0], 0.0), ([2.0 ** -1074] * 3, 0.0),
                       ([2.0 ** 511, 2.0 ** 511], np.inf)):
        a = np.array(vals * 501, dtype=np.float64)  # long enough for several lanes
        K.norm2(dev(a), out, sc)
        got = host(out)[0]
        _, ref = orc.bs3(a, fmad=1)
        if np.isnan(want):
            assert np.isnan(got) and np.isnan(ref)
        else:
            assert got == ref or abs(got - ref) <= 1e-14 * ref, (vals, got, ref)
    # n = 0: the sum is 0.0
    K.norm2(torch.zeros(1, dtype=torch.float64, device="cuda")[:0], out, sc)
    assert host(out)[0] == 0.0


@pytest.mark.parametrize("n", [1, 5, 1000, 65537, 1 << 22])
def test_fast_reductions_fp32_storage(cuda, orc, n):
    a = orc.uniform(n, 1000 + n)
    b = orc.uniform(n, 1100 + n)
    a32, b32 = a.astype(np.float32), b.astype(np.float32)
    sc = K.ReduceScratch()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    K.norm2(dev(a32), out, sc)
    ref = orc.dot_dd(a32, a32)  # FP64 oracle on the stored FP32 values
    assert abs(host(out)[0] - ref) <= 1e-6 * ref
    K.dot(dev(a32), dev(b32), out, sc)
    ref = orc.dot_dd(a32, b32)
    scale = float(np.abs(a32.astype(np.float64) * b32).sum())
    assert abs(host(out)[0] - ref) <= 1e-6 * max(abs(ref), 1e-3 * scale)


@pytest.mark.parametrize("n", [1, 2, 3, 1001, 65536, (1 << 21) + 1])
def test_cg_update_fp64(cuda, orc, n):
    x, r, p, Ap = (orc.uniform(n, s + n) for s in (1, 2, 3, 4))
    alpha = 0.318309886
    dx, dr = dev(x), dev(r)
    sc = K.ReduceScratch()
    rr = torch.zeros(1, dtype=torch.float64, device="cuda")
    K.cg_update(alpha, dev(p), dev(Ap), dx, dr, rr, sc)
    xr, rref, rrref = orc.cg_update(alpha, p, Ap, x, r)
    np.testing.assert_array_equal(host(dx), xr)
    np.testing.assert_array_equal(host(dr), rref)
    # r.r on the integer-pipe accumulator: within 4 ulps of the double-double sum
    assert abs(host(rr)[0] - rrref) <= 4 * np.spacing(rrref)


@pytest.mark.parametrize("n", [1, 3, 4, 1001, 65536, (1 << 21) + 3])
def test_cg_update_fp32_storage(cuda, orc, n):
    x, r, p, Ap = (orc.uniform(n, 10 * s + n).astype(np.float32) for s in (1, 2, 3, 4))
    alpha = 0.318309886
    dx, dr = dev(x), dev(r)
    sc = K.ReduceScratch()
    rr = torch.zeros(1, dtype=torch.float64, device="cuda")
    K.cg_update(alpha, dev(p), dev(Ap), dx, dr, rr, sc)
    xr, rref, rrref = orc.cg_update(np.float32(alpha), p, Ap, x, r)
    np.testing.assert_array_equal(host(dx), xr)
    np.testing.assert_array_equal(host(dr), rref)
    assert abs(host(rr)[0] - rrref) <= 1e-6 * rrref


@pytest.mark.parametrize("n", [1, 2, 5, 1001, 65536, (1 << 21) + 3])
@pytest.mark.parametrize("f32", [False, True])
def test_cg_update_reference_form(cuda, orc, n, f32):
    """r += alpha Ap (bit-exact fma / fmaf) and r.r (FP64 within 4 ulps of the
    double-double sum; FP32 storage 1e-6) in one launch."""
    r, Ap = (orc.uniform(n, 20 * s + n) for s in (1, 2))
    if f32:
        r, Ap = r.astype(np.float32), Ap.astype(np.float32)
    alpha = 0.318309886
    dr = dev(r)
    sc = K.ReduceScratch()
    rr = torch.zeros(1, dtype=torch.float64, device="cuda")
    K.cg_update_ref(alpha, dev(Ap), dr, rr, sc)
    # the oracle's full update with -alpha leaves r = fma(alpha, Ap, r)
    a = np.float32(-alpha) if f32 else -alpha
    _, rref, rrref = orc.cg_update(a, Ap, Ap, np.zeros_like(r), r)
    np.testing.assert_array_equal(host(dr), rref)
    if f32:
        assert abs(host(rr)[0] - rrref) <= 1e-6 * rrref
    else:  # integer-pipe accumulator: within 4 ulps of the double-double sum
        assert abs(host(rr)[0] - rrref) <= 4 * np.spacing(rrref)


def test_bs0_and_graph(cuda):
    a = torch.zeros(1, dtype=torch.float64, device="cuda")
    b = torch.full((1,), 5.0, dtype=torch.float64, device="cuda")
    K.bs0(1, a, b)
    g = K.Bs0Graph(100, 1, a, b)
    g.launch()
    assert host(b)[0] == 5.0  # n != 0: no store
    K.bs0(0, a, b)
    assert host(b)[0] == 0.0  # n == 0: the guarded store happens
