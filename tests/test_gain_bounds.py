"""The regression scans evaluate the float-float variance gain only where the
cheap bounds of variance_gain_bounds (csrc/dml_device.cuh) allow it to reach
the best, so those bounds must hold for every input the engine can see:
lo <= variance_gain <= hi.  This restates the bounds' float32 arithmetic in
numpy (round to nearest, like the device intrinsics; __fdividef's 2-ulp error
taken at its worst, against each bound) and checks them against the oracle's
variance_gain, which the GPU parity tests match bit for bit, on random and
adversarial (near-equal means, extreme scales and counts) inputs."""
import numpy as np
import pytest

import oracle

f32 = np.float32


def _bounds(nL, SL, nR, SR, S):
    n = nL + nR
    a, b = nL.astype(f32), nR.astype(f32)
    t1 = SL.astype(f32) * b
    t2 = SR.astype(f32) * a
    d = np.abs(t1 - t2)
    e = (np.abs(t1) + np.abs(t2)) * f32(2.0 ** -20)
    ab = a * b
    rc = f32(1.0) / n.astype(f32)
    w = ab * rc
    # __fdividef: within 2 ulp of the quotient; each bound takes its worst side
    du = (d + e).astype(np.float64) / ab.astype(np.float64)
    dl = np.maximum(d - e, f32(0.0)).astype(np.float64) / ab.astype(np.float64)
    du = du.astype(f32)
    dl = dl.astype(f32)
    for _ in range(3):
        du = np.nextafter(du, f32(0.0))
        dl = np.nextafter(dl, f32(np.inf))
    p2 = np.array([2.0 ** (-2 * s) for s in S], np.float64).astype(f32)
    hi = du * du * w * f32(1.0 + 2.0 ** -16) * p2
    lo = dl * dl * w * f32(1.0 - 2.0 ** -16) * p2
    return lo, hi


def _cases(rng, count):
    """(nL, SL, nR, SR, S) as the engine forms them: a tree draws N rows, the
    target scale S = 61 - ey - ceil(log2 N) keeps |q| <= 2^(61 - ceil(log2 N))."""
    out = []
    for _ in range(count):
        N = int(rng.choice([2, 7, 100, 4601, 1 << 16, 1_000_000, 4_000_000, (1 << 27) - 1]))
        en = int(np.ceil(np.log2(N)))
        ey = int(rng.integers(-80, 100))
        S = 61 - ey - en
        if not -60 <= S <= 62:
            continue
        qmax = 2 ** (61 - en)
        n = int(rng.integers(2, N + 1)) if N > 2 else 2
        nL = int(rng.integers(1, n))
        nR = n - nL
        kind = rng.integers(0, 4)
        mL = float(rng.uniform(-1, 1)) * qmax
        if kind == 0:
            mR = float(rng.uniform(-1, 1)) * qmax
        elif kind == 1:  # near-equal means: heavy cancellation
            mR = mL * (1.0 + float(rng.normal(0, 1e-9)))
        elif kind == 2:  # equal means up to the integer sums
            mR = mL
        else:  # small targets
            mL, mR = float(rng.normal(0, 3)), float(rng.normal(0, 3))
        SL = int(np.clip(round(mL * nL), -qmax * nL, qmax * nL))
        SR = int(np.clip(round(mR * nR), -qmax * nR, qmax * nR))
        out.append((nL, SL, nR, SR, S, int(kind)))
    return out


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_variance_gain_bounds_hold(seed):
    rng = np.random.default_rng(seed)
    cases = _cases(rng, 6000)
    nL = np.array([c[0] for c in cases], np.int64)
    SL = np.array([c[1] for c in cases], np.int64)
    nR = np.array([c[2] for c in cases], np.int64)
    SR = np.array([c[3] for c in cases], np.int64)
    S = [c[4] for c in cases]
    kind = np.array([c[5] for c in cases])
    g = np.array([oracle.variance_gain(*c[:5])[0] for c in cases], np.float32)
    with np.errstate(over="ignore", under="ignore"):
        lo, hi = _bounds(nL, SL, nR, SR, S)
    bad = np.nonzero(~((lo <= g) & (g <= hi)))[0]
    assert bad.size == 0, [(cases[i], lo[i], g[i], hi[i]) for i in bad[:5]]
    # the filter is worth its cost only if the bounds are tight where the means
    # differ (independent means): the median width is near 2^-15 of the gain,
    # and within 2^-10 for almost all cases (means that happen to lie close
    # give wider bounds)
    sel = (kind == 0) & (g > 0) & np.isfinite(hi)
    width = (hi[sel].astype(np.float64) - lo[sel]) / g[sel]
    assert sel.sum() > 500 and np.median(width) < 2.0 ** -13
    assert (width < 2.0 ** -10).mean() > 0.98


def test_target_weight_packing_is_lossless():
    """qw_pack (csrc/dml_device.cuh): q * 2^wb + w in an int64, wb the bit
    length of N, for every weight 0..N a tree can give an entry and every
    target the scale allows, |q| <= 2^(61 - ceil(log2 N)); unpacked by the
    low wb bits and an arithmetic shift."""
    for N in [2, 3, 4, 5, 4601, 1 << 16, (1 << 16) + 1, 1_000_000, 4_000_000, (1 << 27) - 1]:
        wb = N.bit_length()
        qmax = 2 ** (61 - (N - 1).bit_length())
        for q in (qmax, -qmax, qmax - 1, -qmax + 1, 0, 1, -1):
            for w in (0, 1, 2, N - 1, N):
                x = q * (1 << wb) + w
                assert -(1 << 63) <= x < (1 << 63)
                assert x & ((1 << wb) - 1) == w and x >> wb == q
