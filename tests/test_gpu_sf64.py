"""The FP64 kernels' integer-pipe arithmetic (fvh_sf64.cuh) against IEEE
binary64, through fvh_debug_sf64.

Multiply, add, subtract and divide must return the same bits as the FP64
instructions (ops 4..7 of the same entry point) and as the host's IEEE
arithmetic (numpy), for every input: operand classes that take the integer
path (normal operands and results, zeros) and those that go to the hardware
(subnormals, infinities, NaNs, overflow and underflow).  The optimistic
multiply and divide the kernels use (ops 8 and 9, with their FP64 redo) and
their halving of a value (op 10) are held to the same bar.  NaN results are compared as NaN, whatever their
payload.
"""
import numpy as np
import pytest

import flecsale_gb300.hydro as H

pytestmark = pytest.mark.gpu

N = 1 << 21
SIGN = np.uint64(1 << 63)
MANT = np.uint64((1 << 52) - 1)


def _compose(sign, exp, mant):
    return ((sign.astype(np.uint64) << np.uint64(63)) | (exp.astype(np.uint64) << np.uint64(52))
            | (mant.astype(np.uint64) & MANT)).view(np.float64)


def _operands(mode: int, rng):
    u = lambda: rng.integers(0, 2 ** 63, N, dtype=np.uint64) * np.uint64(2) + \
        rng.integers(0, 2, N, dtype=np.uint64)
    sa, sb = rng.integers(0, 2, N), rng.integers(0, 2, N)
    if mode == 0:  # raw bit patterns: every class, specials included
        return u().view(np.float64), u().view(np.float64)
    if mode == 1:  # exponents within +-3 of each other, around 1
        e0 = 1023 - 40 + rng.integers(0, 81, N)
        return (_compose(sa, e0 + rng.integers(-3, 4, N), u()),
                _compose(sb, e0 + rng.integers(-3, 4, N), u()))
    if mode == 2:  # exponent differences 0..70 (alignment, sticky bits)
        ea = 900 + rng.integers(0, 200, N)
        a = _compose(sa, ea, u())
        b = _compose(sb, ea - rng.integers(0, 71, N), u())
        sw = rng.integers(0, 2, N).astype(bool)
        a[sw], b[sw] = b[sw].copy(), a[sw].copy()
        return a, b
    if mode == 3:  # near-equal magnitudes: cancellation in add/sub
        a = _compose(sa, 1000 + rng.integers(0, 50, N), u())
        delta = rng.integers(-2048, 2048, N)
        big = rng.integers(0, 2, N).astype(bool)
        delta[big] = rng.integers(-(1 << 39), 1 << 39, int(big.sum()))
        bb = (a.view(np.uint64) & ~SIGN).astype(np.int64) + delta
        b = (bb.astype(np.uint64) | (sb.astype(np.uint64) << np.uint64(63))).view(np.float64)
        return a, b
    if mode == 4:  # runs of ones and zeros; exact products and quotients
        ones = MANT >> rng.integers(0, 52, N).astype(np.uint64)
        pow2 = np.uint64(1) << rng.integers(0, 52, N).astype(np.uint64)
        ma = np.where(rng.integers(0, 2, N).astype(bool), ones, pow2)
        a = _compose(sa, 1000 + rng.integers(0, 50, N), ma)
        b = _compose(np.zeros(N, int), 1000 + rng.integers(0, 50, N), u())
        exact = rng.integers(0, 2, N).astype(bool)
        a[exact] = b[exact] * rng.integers(1, 1000, int(exact.sum())).astype(np.float64)
        return a, b
    if mode == 5:  # every exponent (overflow, underflow and subnormal results)
        return (_compose(sa, rng.integers(1, 2047, N), u()),
                _compose(sb, rng.integers(1, 2047, N), u()))

    # mode 6: signed zeros against every class (zeros, normals, subnormals,
    # infinities, NaNs), and pairs of them
    def mix(sign):
        kind = rng.integers(0, 6, N)
        exp = np.select([kind == 0, kind == 1, kind == 2, kind == 3],
                        [np.zeros(N, int), 1023 + rng.integers(-30, 30, N), np.zeros(N, int),
                         np.full(N, 2047)], np.full(N, 2047))
        mant = np.where((kind == 0) | (kind == 3), np.uint64(0), u())
        mant = np.where(kind >= 4, mant | np.uint64(1), mant)  # NaN payloads
        mant = np.where(kind == 2, mant | np.uint64(1), mant)  # subnormals
        return _compose(sign, exp, mant)
    return mix(sa), mix(sb)


def _same(x, y):
    nan = np.isnan(x) & np.isnan(y)
    return nan | (x.view(np.uint64) == y.view(np.uint64))


@pytest.mark.parametrize("mode", range(7))
def test_integer_pipe_arithmetic_is_ieee(cuda, mode):
    torch = cuda
    rng = np.random.default_rng(100 + mode)
    a, b = _operands(mode, rng)
    da, db = torch.tensor(a, device="cuda"), torch.tensor(b, device="cuda")
    out = torch.empty(N, dtype=torch.float64, device="cuda")
    L = H.lib()
    with np.errstate(all="ignore"):
        host = [a * b, a + b, a - b, a / b]
    # ops 0..3 integer pipes, 4..7 FP64 instructions, 8 and 9 the optimistic
    # multiply and divide of the kernels with their FP64 redo
    for op, pair in ((0, (0, 4)), (1, (1, 5)), (2, (2, 6)), (3, (3, 7)), (0, (8, 4)), (3, (9, 7))):
        got = []
        for o in pair:
            H.check(L.fvh_debug_sf64(o, da.data_ptr(), db.data_ptr(), N, out.data_ptr(), None))
            torch.cuda.synchronize()
            got.append(out.cpu().numpy().copy())
        bad = ~_same(got[0], got[1])
        assert not bad.any(), (pair, a[bad][:4], b[bad][:4], got[0][bad][:4], got[1][bad][:4])
        bad = ~_same(got[0], host[op])
        assert not bad.any(), (pair, a[bad][:4], b[bad][:4], got[0][bad][:4], host[op][bad][:4])
    # op 10: the kernels' exact halving (0.5 * a and a / 2 are one value)
    # against the host's 0.5 * a, on every operand class (tiny halves round)
    H.check(L.fvh_debug_sf64(10, da.data_ptr(), db.data_ptr(), N, out.data_ptr(), None))
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    with np.errstate(all="ignore"):
        want = a * 0.5
        assert np.array_equal(want, a / 2, equal_nan=True)
    bad = ~_same(got, want)
    assert not bad.any(), (a[bad][:4], got[bad][:4], want[bad][:4])
