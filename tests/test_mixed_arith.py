"""CPU checks of the FP32 arithmetic the mixed engine uses in place of FP64
instructions (GB300 runs FP64 arithmetic and every 64-bit conversion on a
narrow pipe), restated with numpy's IEEE float32 operations:

* the fixed-point quantisation's split of f = c * 2^sh into h * 2^31 + r
  (`quant`, csrc/mpm_batch_kernels.cuh) gives round-to-nearest-even of f,
  the integer `__float2ll_rn` gives, for |f| <= 2^53;
* the SGMP dual-grid decisions in double-float arithmetic (`sg_locate_df`)
  are the FP64 routines' decisions (cell_of, the half-cell rule for the
  nearest node, dual_cell) whenever they are taken, i.e. outside the 2^-40
  band about a cell face or half cell.
"""
import numpy as np

f32 = np.float32


def _rne_int(x: np.ndarray) -> np.ndarray:
    """Round to nearest even of float64 values holding float32 values
    (exact in float64), as Python integers."""
    return [int(np.rint(v)) for v in x.astype(np.float64)]


def _quant_split(f: np.ndarray) -> list:
    M = f32(1.5 * 2.0**54)
    t = (f + M).astype(f32)  # float32 sum, rounded to nearest even
    h = t.view(np.int32).astype(np.int64) - np.array([M], dtype=f32).view(np.int32).astype(np.int64)[0]
    r = (f - (t - M).astype(f32)).astype(f32)
    lo = np.rint(r.astype(np.float64)).astype(np.int64)  # 32-bit conversion, ties to even
    return [int(a) * 2**31 + int(b) for a, b in zip(h, lo)]


def test_quant_split_equals_round_to_nearest_even():
    rng = np.random.default_rng(7)
    e = rng.integers(-30, 53, size=200_000)
    f = (rng.uniform(-1.0, 1.0, size=e.size) * np.exp2(e.astype(np.float64))).astype(f32)
    ties = np.array([0.5, 1.5, 2.5, -0.5, -1.5, -2.5, 2.0**31, 2.0**30, -(2.0**30), 3 * 2.0**31,
                     5 * 2.0**31, -3 * 2.0**31, 2.0**53, -(2.0**53), 1.5 * 2.0**52, 0.0], dtype=f32)
    f = np.concatenate([f, ties])
    assert np.all(np.abs(f.astype(np.float64)) <= 2.0**53)
    assert _quant_split(f) == _rne_int(f)


# ------------------------------------------------------------ SGMP decisions
def _split(x: np.ndarray):
    """x (float64) as hi (its leading 24 bits) + lo (the rest rounded)."""
    bits = x.view(np.uint64)
    hi = (bits & ~np.uint64((1 << 29) - 1)).view(np.float64).astype(f32)  # truncation to 24 bits: exact
    lo = (x - hi.astype(np.float64)).astype(f32)
    return hi, lo


def _fma32(a, b, c):
    # a * b is exact in float64; the sum is rounded once more to float32
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(f32)


def _df_diff(xh, xl, sh, sl):
    s = (xh - sh).astype(f32)
    bb = (s - xh).astype(f32)
    err = ((xh - (s - bb).astype(f32)).astype(f32) + (-sh - bb).astype(f32)).astype(f32)
    t = (err + (xl - sl).astype(f32)).astype(f32)
    dh = (s + t).astype(f32)
    dl = (t - (dh - s).astype(f32)).astype(f32)
    return dh, dl


def _sg_decisions_df(x, span0, span1, idcell, nc):
    """Per position: taken (bool), cell, nearest node, dual index per axis."""
    xh, xl = _split(x)
    s0h, s1h, ih = f32(span0), f32(span1), f32(idcell)
    s0l, s1l, il = f32(span0 - float(s0h)), f32(span1 - float(s1h)), f32(idcell - float(ih))
    dh, dl = _df_diff(xh, xl, s0h, s0l)
    eh, el = _df_diff(xh, xl, s1h, s1l)
    gtol = (f32(2.0**-40) * np.abs(xh)).astype(f32)
    ok = (dh > gtol) & (eh < -gtol)
    uh = (dh * ih).astype(f32)
    ul = (_fma32(dh, np.full_like(dh, ih), -uh) + _fma32(dh, np.full_like(dh, il), (dl * ih).astype(f32))).astype(f32)
    cf = np.floor(uh).astype(f32)
    fh = (uh - cf).astype(f32)
    r0 = (fh + ul).astype(f32)
    r1 = ((fh - f32(1)).astype(f32) + ul).astype(f32)
    rh = ((fh - f32(0.5)).astype(f32) + ul).astype(f32)
    tol = (f32(2.0**-40) * np.maximum(f32(1), uh)).astype(f32)
    ok &= (r0 > tol) & (r1 < -tol) & (np.abs(rh) > tol)
    c = cf.astype(np.int64)
    ok &= c < nc
    nd = c + (rh > 0)
    dc = np.maximum(nd - 1, 0)
    return ok, c, nd, dc


def _sg_decisions_fp64(x, span0, idcell):
    u = (x - span0) * idcell
    c = np.trunc(u).astype(np.int64)
    nd = c + ((u - c) >= 0.5)
    dc = np.trunc((x - span0) * idcell - 0.5).astype(np.int64)
    return c, nd, dc


def test_sgmp_double_float_decisions_are_the_fp64_ones():
    rng = np.random.default_rng(11)
    span0, dcell, nc = -0.37, 0.0125, 800
    span1 = span0 + nc * dcell
    idcell = 1.0 / dcell
    k = rng.integers(0, nc, size=100_000)
    # uniform positions, positions within 1e-9 .. 1e-15 cells of faces and
    # half cells (either side), and exact half cells
    u = np.concatenate([
        rng.uniform(0.0, nc, size=100_000),
        k + rng.choice([0.0, 0.5, 1.0], size=k.size) + rng.choice([-1, 1], size=k.size) *
        10.0 ** rng.uniform(-15, -9, size=k.size),
        k + 0.5,
    ])
    x = span0 + u * dcell
    inside = (x > span0) & (x < span1)
    uniform = np.arange(x.size) < 100_000
    x, uniform = x[inside], uniform[inside]
    ok, c, nd, dc = _sg_decisions_df(x, span0, span1, idcell, nc)
    c64, nd64, dc64 = _sg_decisions_fp64(x, span0, idcell)
    assert ok[uniform].mean() > 0.999  # positions off the boundaries are decided without FP64
    assert ok[~uniform].mean() < 0.5   # most of those within 1e-9 cells of one go to the FP64 routines
    assert np.array_equal(c[ok], c64[ok])
    assert np.array_equal(nd[ok], nd64[ok])
    assert np.array_equal(dc[ok], dc64[ok])
