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
  * band_far (k_decide, band form): hi <= t + dist certainly false.

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
