"""Host replays of the error-bound shortcuts in the CUDA kernels
(coupe_gb300/csrc/kernels.cuh), in numpy float32/float64 arithmetic:

  * fast_bin / grid_map (k_hist): a key whose grid position lies farther than
    the margin from both bin edges is binned by floor(position); checked
    against the exact bin over the sorted cuts (REF32: f32 midpoints; band
    form: f64 midpoints, the x behind each f32 key, and no key in a cut's
    f32 band);
  * imbalance_test / imbalance_within (k_decide): coupe's f64 test
    |(w - ideal) / ideal| <= tol (recursive_bisection.rs:547-551), settled
    from f32 arithmetic when the estimate is clear of tol;
  * band_far (k_decide, band form): hi <= t + dist certainly false;
  * f2_split and the f32-pair Rib key and box shortcuts (point_f2 in
    k_convert): the key RN32 of coupe's f64 basis-change chain, and the box
    of the mapped points, as the f64 chain gives them;
  * k_moments_f2: the f32-pair inertia sums against exactly rounded sums.

Each replay asserts that whenever a shortcut decides, it decides as the
exact expression does.  The GPU parity tests check the kernels end to end.
"""
import numpy as np

F32 = np.float32


def _rd(x):
    f = F32(x)
    return f if float(f) <= x else np.nextafter(f, F32(-np.inf))


def _ru(x):
    f = F32(x)
    return f if float(f) >= x else np.nextafter(f, F32(np.inf))


def _trunc32(x):
    f = F32(x)
    return np.nextafter(f, F32(0)) if abs(float(f)) > abs(x) else f


def _cut_tree(lo, hi, nbk, mid):
    """The cuts in in-order (sorted) sequence, built depth by depth as
    build_sorted_cuts does."""
    nb = 1 << nbk
    cuts = np.zeros(nb - 1, dtype=type(lo))
    for d in range(nbk):
        h = 1 << (nbk - 1 - d)
        r = (2 * np.arange(1 << d) + 1) * h - 1
        a = np.where(r - h < 0, lo, cuts[np.maximum(r - h, 0)])
        b = np.where(r + h >= nb - 1, hi, cuts[np.minimum(r + h, nb - 2)])
        cuts[r] = mid(a.astype(type(lo)), b.astype(type(lo)))
    return cuts


def _margin(M, sc, nb, ulps):
    u = F32(M) * F32(1.1920929e-7) + F32(1.4012985e-45)
    return F32(1.01) * F32(ulps) * u * sc + F32((nb + 1) * 4.7683716e-7) + F32(9.5367432e-7)


def test_fast_bin_margin():
    rng = np.random.default_rng(7)
    fast_total = 0
    with np.errstate(all="ignore"):
        for trial in range(240):
            nbk = int(rng.integers(3, 11))
            nb = 1 << nbk
            band = trial % 2 == 1
            c = 10.0 ** rng.uniform(-6, 6) * rng.choice([-1, 1])
            ext = abs(c) * 10.0 ** (rng.uniform(-5.5, -2.5) if trial % 3 else rng.uniform(-4, 1))
            lo, hi = c, c + ext
            if trial % 7 == 6:
                lo, hi = -abs(c) * rng.random(), abs(c) * rng.random()
            if band:
                cuts = _cut_tree(lo, hi, nbk, lambda a, b: (a + b) / 2.0)
                l = _trunc32(lo)
                w = F32(hi - lo)
                sc = F32(nb) / w
                s = F32(F32(float(l) - lo) * sc)
                M = max(abs(l), abs(_trunc32(hi)))
                ulps = 1.0
            else:
                lo, hi = F32(lo), F32(hi)
                if not hi > lo:
                    continue
                cuts = _cut_tree(lo, hi, nbk, lambda a, b: (a + b) / F32(2))
                l, sc, s = lo, F32(nb) / F32(hi - lo), F32(0)
                M = max(abs(lo), abs(hi))
                ulps = 0.5 * nbk
            if not (np.isfinite(sc) and np.isfinite(s)):
                continue
            m = _margin(M, sc, nb, ulps)
            if not m < 0.25:
                continue
            xs = list(rng.uniform(float(lo), float(hi), 4000))
            step = max(1, len(cuts) // 48)
            for cc in cuts[::step]:
                k = F32(cc)
                for _ in range(3):
                    xs += [float(k), float(np.nextafter(k, F32(np.inf))), float(np.nextafter(k, F32(-np.inf)))]
                    k = np.nextafter(k, F32(np.inf))
                if band:
                    xs += [float(cc), float(np.nextafter(float(cc), np.inf)), float(np.nextafter(float(cc), -np.inf))]
            x = np.asarray(xs)
            k = x.astype(F32)
            keep = (k >= _rd(float(lo))) & (k <= _ru(float(hi)))
            x, k = x[keep], k[keep]
            f = (k.astype(np.float64) - float(l)) * float(sc) + float(s)   # fused multiply-add, rounded once
            f = f.astype(F32)
            bg = np.trunc(f).astype(np.int64)
            fr = f - bg.astype(F32)
            fast = (bg >= 0) & (bg < nb) & (fr > m) & (fr < F32(1) - m)
            fast_total += int(fast.sum())
            if band:
                exact = np.searchsorted(cuts, x[fast], side="right")
                lob = np.array([_rd(float(cc)) for cc in cuts])
                hib = np.array([_ru(float(cc)) for cc in cuts])
                kf = k[fast]
                j = np.searchsorted(lob, kf, side="right") - 1   # the last cut whose band starts at or below k
                in_band = (j >= 0) & (hib[np.maximum(j, 0)] >= kf)
                assert not in_band.any()
            else:
                exact = np.searchsorted(cuts, k[fast], side="right")
            np.testing.assert_array_equal(bg[fast], exact)
    assert fast_total > 100_000


def test_imbalance_shortcut():
    rng = np.random.default_rng(1)
    decided = 0
    with np.errstate(all="ignore"):
        for it in range(40_000):
            if it % 2:
                ideal = float(rng.standard_normal() * 10.0 ** rng.integers(-30, 30))
            else:
                ideal = float(int(rng.integers(-2 ** 62, 2 ** 62))) / 2.0
            if ideal == 0.0:
                continue
            tol = float(rng.choice([0.01, 0.05, 0.005, 1e-7, 1e-9, 0.3, 1.0, -1.0, rng.random()]))
            idf = F32(ideal)
            a = abs(idf)
            if not (F32(2.0 ** -100) <= a <= F32(2.0 ** 100)):
                continue
            rinv = F32(1) / a
            tlo, thi = _rd(tol), _ru(tol)
            rel = rng.choice([-1, 1]) * tol * (1 + rng.standard_normal(4) * 10.0 ** -rng.integers(3, 8))
            cands = [ideal * (1 + r) for r in rel] + [ideal * rng.standard_normal() * 3]
            for w in cands:
                exact = abs((w - ideal) / ideal) <= tol
                wf = F32(w)
                q = abs(wf - idf) * rinv
                e = F32(2.0 ** -21) * ((abs(wf) + abs(idf)) * rinv + q)
                up, dn = q + e, q - e
                if up <= tlo and up <= F32(2.0 ** 127):
                    decided += 1
                    assert exact, (w, ideal, tol)
                elif dn > thi:
                    decided += 1
                    assert not exact, (w, ideal, tol)
    assert decided > 50_000


def test_band_far_shortcut():
    rng = np.random.default_rng(2)
    far_count = 0
    with np.errstate(all="ignore"):
        for it in range(60_000):
            sc = 10.0 ** rng.integers(-20, 20)
            t = float(rng.standard_normal() * sc)
            mode = it % 4
            if mode == 0:
                x = t + abs(rng.standard_normal()) * sc * 10.0 ** rng.integers(-12, 1)
            elif mode == 1:
                x = t + abs(t) * 2.0 ** -int(rng.integers(20, 60))
            elif mode == 2:
                x = t
            else:
                x = float(rng.standard_normal() * sc)
            k = F32(x)
            if not np.isfinite(k):
                continue
            kd = float(k)
            xl = (kd + float(np.nextafter(k, F32(-np.inf)))) / 2.0
            xh = (kd + float(np.nextafter(k, F32(np.inf)))) / 2.0
            if rng.random() < 0.3:
                xl = xh = min(max(x, xl), xh)  # an exact minimum found by a pass
            xl = max(xl, t)
            xh = max(xh, xl)
            dl, dh = xl - t, xh - t
            r = rng.random()
            if r < 0.3:
                hi = t + dh
            elif r < 0.5:
                hi = float(np.nextafter(t + dh, np.inf))
            else:
                hi = t + abs(rng.standard_normal()) * sc * 10.0 ** rng.integers(-15, 3)
            if hi < t:
                continue
            tlo, thi, hlo = _rd(t), _ru(t), _rd(hi)
            nk = np.nextafter(k, F32(np.inf))
            M = max(nk, thi)
            A = max(abs(M), abs(tlo))
            if not all(np.isfinite(v) for v in (k, nk, tlo, M, A)):
                continue
            bound = _ru(float(M) + float(_ru(float(A) * 2.0 ** -50)))
            if hlo > bound:
                far_count += 1
                assert not (hi <= t + dl) and not (hi <= t + dh), (k, t, hi)
    assert far_count > 5_000


# ---------------------------------------------------------------- f32 pairs
def _f2_split(x):
    """f2_split (common.cuh): hi = RN32(x), lo = RN32(x - hi), from the f64
    fields with integer operations."""
    import struct
    b = struct.unpack("<Q", struct.pack("<d", x))[0]
    e = (b >> 52) & 0x7FF
    if (b << 1) & 0xFFFFFFFFFFFFFFFF == 0:
        return F32(0), F32(0)
    if not 1023 - 50 <= e <= 1023 + 50:
        return None  # the kernels take the f64 path
    M = (b & ((1 << 52) - 1)) | (1 << 52)
    H = (M + 0x0FFFFFFF + ((M >> 29) & 1)) >> 29
    R = M - (H << 29)
    sh = np.frombuffer(struct.pack("<I", (e - 1046 + 127) << 23), dtype=F32)[0]
    sl = np.frombuffer(struct.pack("<I", (e - 1075 + 127) << 23), dtype=F32)[0]
    h, l = F32(F32(H) * sh), F32(F32(R) * sl)
    return (-h, -l) if b >> 63 else (h, l)


def test_f2_split_matches_rounding():
    rng = np.random.default_rng(3)
    for it in range(20_000):
        x = float(rng.standard_normal() * 2.0 ** rng.integers(-49, 49))
        if it % 7 == 0:
            x = float(F32(x)) * (1 + 2.0 ** -24)  # halfway cases
        r = _f2_split(x)
        if r is not None:
            assert r[0] == F32(x) and r[1] == F32(x - float(F32(x)))


def _pair_ops():
    def two_sum(a, b):
        s = F32(a + b)
        v = F32(s - a)
        return s, F32((a - (s - v)) + (b - v))

    def fast(a, b):
        s = F32(a + b)
        return s, F32(b - (s - a))

    def fma(a, b, c):
        return F32(np.float64(a) * np.float64(b) + np.float64(c))

    def mul(a, b):
        p = F32(a[0] * b[0])
        e = fma(a[0], b[0], -p)
        e = fma(a[0], b[1], e)
        e = fma(a[1], b[0], e)
        return fast(p, e)

    def add(acc, x):
        s = two_sum(acc[0], x[0])
        return fast(s[0], F32(s[1] + F32(acc[1] + x[1])))
    return mul, add


def test_rib_key_shortcut():
    """point_f2 (k_convert): the key RN32 of coupe's f64 chain
    ((m0 p0 + m1 p1) + m2 p2) is the pair estimate's high part whenever no
    f32 rounding boundary lies within the bound of it."""
    mul, add = _pair_ops()
    rng = np.random.default_rng(5)
    fast_n = 0
    for trial in range(12):
        D = 3 if trial % 2 == 0 else 2
        Q, _ = np.linalg.qr(rng.standard_normal((D, D)))
        sc = 10.0 ** rng.uniform(-3, 5)
        for _ in range(400):
            p = rng.standard_normal(D) * sc * np.array([1, 10, 100][:D])
            if trial % 3 == 0:
                p = np.round(p, 2)
            pp = [_f2_split(float(v)) for v in p]
            if any(v is None for v in pp):
                continue
            for r in range(D):
                y = Q[r, 0] * p[0]
                for c in range(1, D):
                    y = y + Q[r, c] * p[c]
                m = [_f2_split(float(v)) for v in Q[r]]
                if any(v is None for v in m):
                    continue
                acc = mul(m[0], pp[0])
                sabs = F32(abs(F32(m[0][0] * pp[0][0])))
                for c in range(1, D):
                    acc = add(acc, mul(m[c], pp[c]))
                    sabs = F32(sabs + abs(F32(m[c][0] * pp[c][0])))
                e = F32(sabs * F32(2.0 ** -39))
                hb = int(np.asarray(acc[0], dtype=F32).view(np.uint32))
                ex = (hb >> 23) & 0xFF
                if not 25 <= ex <= 253:
                    continue
                u = np.frombuffer(np.uint32((ex - 23) << 23).tobytes(), dtype=F32)[0]
                up = F32(0.5) * u
                down = F32(0.5) * u if hb & 0x7FFFFF else F32(0.25) * u
                away = -acc[1] if hb >> 31 else acc[1]
                if F32(away + e) < up and F32(e - away) < down:
                    fast_n += 1
                    assert acc[0] == F32(y), (p, r)
    assert fast_n > 5_000


def test_rib_box_shortcut():
    """point_f2's box test: a point is skipped only when its bounds lie
    strictly inside the f32 bounds of the running exact box; the box found
    equals the exact one, also for sorted and tied values."""
    rng = np.random.default_rng(9)
    for trial in range(12):
        n = 3000
        y = rng.standard_normal(n) * 10.0 ** rng.uniform(-3, 6)
        if trial % 3 == 0:
            y = np.sort(y)
        if trial % 3 == 1:
            y = np.round(y, 1)
        e = np.abs(y) * 2.0 ** -40 * rng.uniform(0.5, 4, n)
        est = y + rng.uniform(-1, 1, n) * e * 0.9
        yh = est.astype(F32)
        yl = (est - yh.astype(np.float64)).astype(F32)
        ef = e.astype(F32)
        mn, mx, mnf, mxf = np.inf, -np.inf, F32(np.inf), F32(-np.inf)
        for i in range(n):
            slack = F32(F32(abs(yl[i]) + ef[i]) + F32(abs(yh[i]) * F32(2.0 ** -22)))
            if F32(yh[i] - slack) > mnf and F32(yh[i] + slack) < mxf:
                continue
            mn, mx = min(mn, y[i]), max(mx, y[i])
            mnf = np.nextafter(F32(mn), F32(np.inf))
            mxf = np.nextafter(F32(mx), F32(-np.inf))
        assert mn == y.min() and mx == y.max()


def test_pair_inertia_sums_accuracy():
    """k_moments_f2: the unweighted Rib sums (offsets from the first point,
    their sums and products) in f32-pair arithmetic, one thread's sequence
    at a time, match exactly rounded sums to 1e-12 relative."""
    from math import fsum
    mul, add = _pair_ops()
    rng = np.random.default_rng(0)
    side = 24
    g = np.arange(side) + 0.5
    x, y, z = np.meshgrid(g, g * 10, g * 100, indexing="ij")
    q, _ = np.linalg.qr(rng.standard_normal((3, 3)))
    pts = np.stack([x.ravel(), y.ravel(), z.ravel()], 1) @ q.T + 1000.0
    s = [_f2_split(float(v)) for v in pts[0]]
    pairs = [(a, b) for a in range(3) for b in range(a, 3)]
    threads = 64
    S1 = np.zeros(3)
    S2 = np.zeros(len(pairs))
    for t in range(threads):
        a1 = [(F32(0), F32(0))] * 3
        a2 = [(F32(0), F32(0))] * len(pairs)
        for p in pts[t::threads]:
            o = []
            for d in range(3):
                ph, pl = _f2_split(float(p[d]))
                sh = F32(ph + F32(-s[d][0]))
                v = F32(sh - ph)
                err = F32(F32(ph - F32(sh - v)) + F32(F32(-s[d][0]) - v))
                t2 = F32(err + F32(pl - s[d][1]))
                hi = F32(sh + t2)
                o.append((hi, F32(t2 - F32(hi - sh))))
            a1 = [add(a1[d], o[d]) for d in range(3)]
            a2 = [add(a2[k], mul(o[i], o[j])) for k, (i, j) in enumerate(pairs)]
        S1 += [float(h) + float(l) for h, l in a1]
        S2 += [float(h) + float(l) for h, l in a2]
    off = pts - pts[0]
    R1 = np.array([fsum(off[:, d]) for d in range(3)])
    R2 = np.array([fsum(off[:, i] * off[:, j]) for i, j in pairs])
    assert np.abs(S1 - R1).max() <= 1e-12 * np.abs(R1).max()
    assert np.abs(S2 - R2).max() <= 1e-12 * np.abs(R2).max()
