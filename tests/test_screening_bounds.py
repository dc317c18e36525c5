"""The error bounds behind two exact-result shortcuts, emulated in numpy on
adversarial inputs (no GPU):

* the query index files a key by floor() of its corners in level-0 cells,
  computed in float with a margin (stc_query.cu, index_file_fast); a key
  whose corner is within the margin of a cell edge takes the exact FP64
  decode. Whenever the float filing is used it must equal the exact one.
* compaction decodes a box coordinate as the float nearest to
  base + (q / qmax) * w in double (stc_compact.cu, parse_coord); the division
  is replaced by a reciprocal whose error is bounded, and the float is kept
  only when both ends of the bound round to it. It must equal the float of
  the exact double expression."""
import numpy as np

f32 = np.float32


def _exact_cells(low0, x, mx, me, m0, wx, le, sx):
    box0 = m0 + (low0 / mx) * wx
    box2 = box0 + (x / me) * le
    return (box0 - m0) * sx, (box2 - m0) * sx


def test_float_index_filing_agrees_with_the_exact_decode():
    rng = np.random.default_rng(1)
    decided = 0
    for _ in range(200):
        m0 = f32(rng.uniform(-180, 180))
        w = f32(10 ** rng.uniform(-6, 0.5))
        m2 = f32(m0 + w)
        wy = f32(10 ** rng.uniform(-6, 0.5))
        wx = f32(m2 - m0)
        if not wx > 0:
            continue
        le = float(max(wx, wy))
        g = int(2 ** rng.integers(4, 9))
        sx = g / (float(m2) - float(m0))
        bl, be = int(rng.integers(4, 33)), int(rng.integers(4, 33))
        mx, me = float((1 << bl) - 1), float((1 << be) - 1)
        # the host's coefficients (index_file_coeffs)
        a, b = sx * float(wx) / mx, sx * le / me
        m = max(abs(float(m0)), abs(float(m2))) + le + 1.0
        d = f32(sx * m * 2.0 ** -46) + f32(1e-9)
        n = 10000
        low0 = rng.integers(0, 1 << bl, n).astype(np.uint64)
        # half of them next to cell edges
        k = rng.integers(0, g + 2, n // 2)
        low0[: n // 2] = np.clip(np.floor(k / a + rng.integers(-2, 3, n // 2)), 0, (1 << bl) - 1).astype(np.uint64)
        x = rng.integers(0, 1 << be, n).astype(np.uint64)
        e0, e1 = _exact_cells(low0.astype(np.float64), x.astype(np.float64), mx, me, float(m0), float(wx), le, sx)
        f0 = low0.astype(np.float32) * f32(a)
        f1 = f0 + x.astype(np.float32) * f32(b)

        def sure(v):
            dd = v * f32(1e-6) + d
            lo, hi = np.floor(v - dd), np.floor(v + dd)
            return lo == hi, lo

        s0, l0 = sure(f0)
        s1, l1 = sure(f1)
        ok = s0 & s1
        decided += int(ok.sum())
        assert not (ok & ((l0 != np.floor(e0)) | (l1 != np.floor(e1)))).any()
    assert decided > 0


def test_reciprocal_box_decode_agrees_with_the_division():
    rng = np.random.default_rng(5)
    kept = 0
    for _ in range(150):
        base = f32(rng.uniform(-180, 180))
        w = f32(10 ** rng.uniform(-6, 1))
        bits = int(rng.integers(2, 33))
        qmax = float((1 << bits) - 1)
        rq = 1.0 / qmax
        # the host's bound (lsm_compact): 2^-46 (|base| + 2|w| + 1)
        d = (abs(float(base)) + 2 * abs(float(w)) + 1.0) * 2.0 ** -46
        n = 20000
        q = rng.integers(0, 1 << bits, n).astype(np.float64)
        # half of them next to float rounding midpoints of the result
        tgt = (np.float64(base) + q * (float(w) / qmax)).astype(np.float32)
        mid = (tgt.astype(np.float64) + np.nextafter(tgt, np.float32(np.inf)).astype(np.float64)) / 2
        q[: n // 2] = np.clip(np.round((mid - float(base)) / float(w) * qmax), 0, qmax)[: n // 2]
        exact = (np.float64(base) + (q / qmax) * np.float64(w)).astype(np.float32)
        v = np.float64(base) + q * rq * np.float64(w)
        lo, hi = (v - d).astype(np.float32), (v + d).astype(np.float32)
        ok = lo == hi
        kept += int(ok.sum())
        assert not (ok & (lo != exact)).any()
    assert kept > 0
