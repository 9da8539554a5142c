"""Soundness of the certified bounds of the precision form, checked on the CPU: the FP32
filter of the survivor pass (ct_screen.cu: warp_dots_f32 + pair_bounds_f32 and the
per-query constants of two_level_topk), the FP32 GEMM filter of the exhaustive pass
(filter_tile_kernel: blocked sums of FMA chains of 16 elements, pair_bounds_core) and the
sweep epilogue's bounds on |rho| for any tensor-core dot within the certified BF16 error
band (screen_sweep_kernel, phase 1).

The kernel's float32 arithmetic is restated operation by operation in numpy: each of the
32 lanes runs an FMA chain over its m/32 contiguous elements, a butterfly of additions
joins them, and the kernel value comes from the scaled f32 coordinates.  __expf is taken
at both ends of its documented error band (2 + floor(1.2 |x|) ulp, a little wider than
the CUDA documentation states).  The test asserts that the FP64 value of d^2 = 1 - |rho|
(the oracle's definition over the stored f32 inputs) lies inside [dl2, du2] for random
pairs, pairs with tiny residual variance (inducing rows) and near-duplicate points, for
both kernels.  A candidate is discarded on these bounds alone, so a bound that misses the
truth would drop a true neighbour.
"""
import numpy as np
import pytest

from oracle import oracle as O

F = np.float32


def fma32(a, b, c):
    # single rounding of a*b + c (the product of two floats is exact in double)
    return F(np.float64(a) * np.float64(b) + np.float64(c))


def expf_band(x):
    e = F(np.exp(np.float64(x)))
    u = int(2 + np.floor(1.2 * abs(float(x))))
    lo = hi = e
    for _ in range(u):
        lo = np.nextafter(lo, F(-np.inf))
        hi = np.nextafter(hi, F(np.inf))
    return (e, lo, hi)


def dot_f32(vq, vc, m):
    per = m // 32
    s = np.zeros(32, dtype=F)
    for lane in range(32):
        acc = F(0.0)
        for t in range(per):
            acc = fma32(vq[lane * per + t], vc[lane * per + t], acc)
        s[lane] = acc
    for off in (16, 8, 4, 2, 1):
        s = np.array([F(s[ln] + s[ln ^ off]) for ln in range(32)], dtype=F)
    return s[0]


def dot_blocked(vq, vc, m, flb=16):
    """filter_tile_kernel's dot: FMA chains of flb consecutive elements, each added to a total."""
    tot = F(0.0)
    for b in range(0, m, flb):
        acc = F(0.0)
        for e in range(b, b + flb):
            acc = fma32(vq[e], vc[e], acc)
        tot = F(tot + acc)
    return tot


def bounds(q, c, data, exp_pick, kind="survivor"):
    """[dl2, du2] of the pair as the kernel computes them (exp_pick: 0 nominal, 1 low, 2 high;
    kind: the survivor pass's lane chains or the exhaustive pass's blocked GEMM sums)."""
    Vf, xs, vn, isp, xmax, xmax_max, var, kt, m, d = data
    if kind == "survivor":
        dot = dot_f32(Vf[q], Vf[c], m)
        ed_q = F(F(F((m >> 5) + 7) * F(5.97e-8)) * vn[q])
    else:
        dot = dot_blocked(Vf[q], Vf[c], m)
        ed_q = F(F(F(16 + m // 16 + 1) * F(5.97e-8)) * vn[q])
    ed = F(ed_q * vn[c])
    dd = F(d)
    ced2 = F(F(dd + F(2.0)) * F(5.97e-8))
    A = F(F(2.4e-7) * F(xmax[q] + xmax_max))
    ale = F(F(ced2 + F(F(F(0.5) * A) * dd)) * F(1.00001))
    bee = F(F(F(0.5) * A) * F(1.00001))
    alk = F(F(F(F(6e-8) + F(F(0.5) * ced2)) + F(F(F(0.25) * A) * dd)) * F(1.00001))
    bek = F(F(F(1e-6) + F(F(0.25) * A)) * F(1.00001))
    d2 = F(0.0)
    for a in range(d):
        t = F(xs[c, a] - xs[q, a])
        d2 = fma32(t, t, d2)
    if kt == 0:
        e = expf_band(F(F(-0.5) * d2))[exp_pick]
        kv = F(F(var) * e)
        ek = F(kv * fma32(alk, d2, bek))
    else:
        ed2 = fma32(ale, d2, bee)
        a = F(F(2.2360679775) * F(np.sqrt(d2)))
        ea = expf_band(F(-a))[exp_pick]
        kv = F(F(F(var) * F(F(F(1.0) + a) + F(F(a * a) * F(0.33333334)))) * ea)
        t1 = F(kv * F(F(1e-6) + F(F(2.4e-7) * a)))
        t2 = F(F(F(F(var) * F(F(F(0.8334) * ed2) + F(F(F(1e-7) * a) * a))) * F(F(1.0) + a)) * ea)
        ek = F(t1 + t2)
    R = F(abs(F(kv - dot)))
    e = F(F(ed + ek) + fma32(R, F(1.2e-7), F(1e-30)))
    sc = min(F(isp[q] * isp[c]), F(1e9))
    rl = F(F(max(F(R - e), F(0.0)) * sc) * F(1.0 - 2e-6))
    rh = F(F(F(R + e) * sc) * F(1.0 + 2e-6))
    du2 = F(1.0) - min(rl, F(1.0))
    dl2 = max(F(1.0) - min(rh, F(1.0)), F(0.0))
    return float(dl2), float(du2)


def _case(n, d, m, kt, ls, seed, dup=8):
    r = np.random.default_rng(seed)
    X = r.standard_normal((n, d)).astype(np.float32)
    # near-duplicates: the last rows copy earlier ones with 1e-4 perturbations
    X[n - dup:] = X[:dup] + F(1e-4) * r.standard_normal((dup, d)).astype(np.float32)
    V, p, idx, _ = O.build_residual_backend_np(X, seed=seed + 1, inducing_count=m, variance=1.0, lengthscale=ls,
                                               kernel_type=kt)
    V = V.astype(np.float32)
    p = p.astype(np.float32)
    xs = (X * F(1.0 / ls)).astype(np.float32)
    vn = np.array([np.nextafter(F(np.sqrt(np.sum(V[i].astype(np.float64) ** 2))), F(np.inf)) for i in range(n)],
                  dtype=np.float32)
    isp = (1.0 / np.sqrt(p.astype(np.float64))).astype(np.float32)
    xmax = np.max(np.abs(xs), axis=1).astype(np.float32)
    data = (V, xs, vn, isp, xmax, F(xmax.max()), 1.0, kt, m, d)
    return X, V, p, idx, data


@pytest.mark.parametrize("kind", ["survivor", "gemm"])
@pytest.mark.parametrize("n,d,m,kt,ls", [
    (1500, 3, 64, 1, 1.0),   # Matern 5/2, serving-like
    (1500, 8, 64, 0, 2.0),   # RBF, precision-workload-like
    (1200, 3, 128, 0, 0.7),  # RBF, short lengthscale, m % 128 == 0 (float4 lane shares)
    (1200, 5, 96, 1, 2.0),   # Matern, m % 128 != 0 (scalar lane shares)
])
def test_fp32_filter_bounds_contain_fp64(n, d, m, kt, ls, kind):
    X, V, p, idx, data = _case(n, d, m, kt, ls, seed=n + d + m)
    r = np.random.default_rng(7)
    pairs = [tuple(r.choice(n, 2, replace=False)) for _ in range(120)]
    pairs += [(int(idx[i]), int(j)) for i, j in zip(range(0, len(idx), max(1, len(idx) // 12)),
                                                      r.choice(n, 12, replace=False))]  # tiny-p queries
    pairs += [(int(j), int(idx[i])) for i, j in zip(range(0, len(idx), max(1, len(idx) // 12)),
                                                      r.choice(n, 12, replace=False))]  # tiny-p candidates
    pairs += [(i, n - 8 + i) for i in range(8)]                                          # near-duplicates
    ls_vec = np.full(d, ls, np.float32)
    widths = []
    for i, (q, c) in enumerate(pairs):
        if q == c:
            continue
        truth = float(O.residual_dist_f64(V, p, X, 1.0, ls_vec, kt, [q], [c])[0, 0]) ** 2
        for pick in (0, 1, 2):
            dl2, du2 = bounds(q, c, data, pick, kind)
            assert dl2 <= truth <= du2, (q, c, pick, dl2, truth, du2)
        if i < 120:
            widths.append(du2 - dl2)
    # not vacuous: the random pairs' bounds are narrow (the filter decides them)
    assert np.median(widths) < 1e-3, np.median(widths)


def epilogue_rho_bounds(q, c, data, v_mma, exp_pick, raw=False):
    """Lower / upper bounds of |rho| the sweep epilogue derives for one pair from a tensor-core
    dot v_mma: the heap uses max(blo, 0) isq (1 - 1e-6), the survivor test bhi isq / (1 - 2e-6)."""
    Vf, xs, vn, isp, xmax, xmax_max, var, kt, m, d = data
    u2 = 1.0 / 65536.0
    err_coef = F(3.1 * u2 + (3.0 * m / 16.0 + 17.0) * 2.0 ** -22)
    err_c = F(err_coef * vn[c])
    vnq, isq, isc = vn[q], isp[q], isp[c]
    dd = F(d)
    ced2 = F(F(dd + F(2.0)) * F(5.97e-8))
    A = F(F(2.4e-7) * F(xmax[q] + xmax_max))
    ale = F(F(ced2 + F(F(F(0.5) * A) * dd)) * F(1.00001))
    bee = F(F(F(0.5) * A) * F(1.00001))
    alk = F(F(F(F(6e-8) + F(F(0.5) * ced2)) + F(F(F(0.25) * A) * dd)) * F(1.00001))
    bek = F(F(F(1e-6) + F(F(0.25) * A)) * F(1.00001))
    d2 = F(0.0)
    for a in range(d):
        t = F(xs[c, a] + F(-xs[q, a]))
        d2 = fma32(t, t, d2)
    if kt == 0:
        e = expf_band(F(F(-0.5) * d2))[exp_pick]
        kv = F(F(var) * e)
        ek = F(kv * fma32(alk, d2, bek))
    else:
        ed2 = fma32(ale, d2, bee)
        a = F(F(2.2360679775) * F(np.sqrt(d2)))
        ea = expf_band(F(-a))[exp_pick]
        kv = F(F(F(var) * F(F(F(1.0) + a) + F(F(a * a) * F(0.33333334)))) * ea)
        t1 = F(kv * F(F(1e-6) + F(F(2.4e-7) * a)))
        t2 = F(F(F(F(var) * F(F(F(0.8334) * ed2) + F(F(F(1e-7) * a) * a))) * F(F(1.0) + a)) * ea)
        ek = F(t1 + t2)
    R = F(abs(F(kv + F(-v_mma))))
    e = F(fma32(vnq, err_c, ek) + fma32(R, F(1.2e-7), F(1e-30)))
    blo = F(F(R + F(-e)) * isc)
    bhi = F(F(R + e) * isc)
    if raw:
        return blo, bhi
    rho_lo = float(F(F(max(blo, F(0.0)) * isq) * F(1.0 - 1e-6)))
    rho_hi = float(bhi) * float(isq) / (1.0 - 2e-6)
    return rho_lo, rho_hi


@pytest.mark.parametrize("n,d,m,kt,ls", [
    (1500, 3, 64, 1, 1.0),
    (1500, 8, 64, 0, 2.0),
    (1200, 3, 128, 0, 0.7),
])
def test_epilogue_bounds_contain_fp64(n, d, m, kt, ls):
    """The sweep's bounds on |rho| for a tensor-core dot anywhere in its certified BF16 error
    band (c_split |v_q| |v_c| around the exact dot) contain the FP64 |rho|."""
    X, V, p, idx, data = _case(n, d, m, kt, ls, seed=n + d + m + 1)
    vn = data[2]
    u2 = 1.0 / 65536.0
    c_split = 3.1 * u2 + (3.0 * m / 16.0 + 17.0) * 2.0 ** -22
    r = np.random.default_rng(11)
    pairs = [tuple(r.choice(n, 2, replace=False)) for _ in range(100)]
    pairs += [(int(idx[i]), int(j)) for i, j in zip(range(0, len(idx), max(1, len(idx) // 10)),
                                                      r.choice(n, 10, replace=False))]
    pairs += [(i, n - 8 + i) for i in range(8)]
    ls_vec = np.full(d, ls, np.float32)
    for q, c in pairs:
        if q == c:
            continue
        rho_true = 1.0 - float(O.residual_dist_f64(V, p, X, 1.0, ls_vec, kt, [q], [c])[0, 0]) ** 2
        exact = float(np.dot(V[q].astype(np.float64), V[c].astype(np.float64)))
        band = c_split * float(vn[q]) * float(vn[c])
        for v_mma in (F(exact), F(exact - band), F(exact + band)):
            for pick in (0, 1, 2):
                lo, hi = epilogue_rho_bounds(q, c, data, v_mma, pick)
                assert lo <= rho_true <= hi, (q, c, float(v_mma), pick, lo, rho_true, hi)


def _query_consts(q, data):
    Vf, xs, vn, isp, xmax, xmax_max, var, kt, m, d = data
    dd = F(d)
    ced2 = F(F(dd + F(2.0)) * F(5.97e-8))
    A = F(F(2.4e-7) * F(xmax[q] + xmax_max))
    ale = F(F(ced2 + F(F(F(0.5) * A) * dd)) * F(1.00001))
    bee = F(F(F(0.5) * A) * F(1.00001))
    alk = F(F(F(F(6e-8) + F(F(0.5) * ced2)) + F(F(F(0.25) * A) * dd)) * F(1.00001))
    bek = F(F(F(1e-6) + F(F(0.25) * A)) * F(1.00001))
    if kt == 0:
        ekmax = F(F(F(var) * F(F(F(0.7358) * alk) + bek)) * F(1.01))
    else:
        ekmax = F(F(F(var) * F(F(F(1.283e-6) + F(F(0.8334) * F(F(F(0.3628) * ale) + bee))) + F(1.82e-7))) * F(1.01))
    return ekmax


def group_hi(q, half, cands, data, v_mmas, kpick):
    """The sweep epilogue's group test (screen_sweep_kernel), float32 operation by operation:
    kmax from the box of the half tile `half` (computed once per job), then a bound on
    phase 1's survivor bound bhi of every pair of the group `cands` (a subset of the half
    tile).  kpick 1 takes __expf at the low end of its error band."""
    Vf, xs, vn, isp, xmax, xmax_max, var, kt, m, d = data
    u2 = 1.0 / 65536.0
    err_coef = F(3.1 * u2 + (3.0 * m / 16.0 + 17.0) * 2.0 ** -22)
    lo = xs[half].min(axis=0)
    hi = xs[half].max(axis=0)
    err_max = max(F(err_coef * vn[c]) for c in cands)
    isc_max = max(isp[c] for c in cands)
    dmin = F(0.0)
    for a_ in range(d):
        a = F(lo[a_] + F(-xs[q, a_]))
        b = F(hi[a_] + F(-xs[q, a_]))
        t = max(max(a, F(-b)), F(0.0))
        dmin = fma32(t, t, dmin)
    dmin = F(dmin * F(1.0 - 1e-5))
    lo_e = 1 if kpick else 0
    if kt == 0:
        kmax = F(F(F(var) * expf_band(F(F(-0.5) * dmin))[lo_e]) * F(1.0 + 1e-5))
    else:
        a0 = F(F(2.2360679775) * F(np.sqrt(dmin)))
        kmax = F(F(F(F(var) * F(F(F(1.0) + a0) + F(F(a0 * a0) * F(0.33333334)))) * expf_band(F(-a0))[lo_e]) * F(1.0 + 2e-5))
    rmax = F(0.0)
    for v in v_mmas:
        rmax = max(rmax, max(F(kmax - v), v))
    ekmax = _query_consts(q, data)
    inner = F(F(F(rmax * F(1.0 + 3e-7)) + F(vn[q] * err_max)) + F(ekmax + F(1e-30)))
    return F(F(inner * isc_max) * F(1.0 + 1e-6))


@pytest.mark.parametrize("n,d,m,kt,ls", [
    (1500, 8, 64, 0, 2.0),   # RBF, precision-workload-like
    (1500, 3, 64, 1, 1.0),   # Matern 5/2
    (1200, 3, 128, 0, 0.7),  # RBF, short lengthscale
    (1200, 5, 96, 1, 2.0),   # Matern, D = 5
])
def test_group_test_bounds_every_pair(n, d, m, kt, ls):
    """The sweep's group test never rejects a group holding a pair that phase 1 would keep
    or heap: its bound is >= phase 1's survivor bound bhi of every pair, for tensor-core dots
    anywhere in the certified band, __expf at either end of its band, for groups of 8 points
    close together (coordinate-sorted, tight boxes), random groups, groups holding the query
    itself and groups with tiny-p rows.  The kernel-value bound comes from the box of the
    group's half tile (128 candidates)."""
    X, V, p, idx, data = _case(n, d, m, kt, ls, seed=n + d + m + 5)
    xs, vn = data[1], data[2]
    u2 = 1.0 / 65536.0
    c_split = 3.1 * u2 + (3.0 * m / 16.0 + 17.0) * 2.0 ** -22
    r = np.random.default_rng(23)
    order = np.lexsort(tuple(xs[:, a] for a in range(d)))  # coordinate-sorted: tight half tiles
    halves = [order[128 * h:128 * h + 128] for h in r.choice(n // 128, 6, replace=False)]
    halves += [r.choice(n, 128, replace=False) for _ in range(3)]
    halves += [np.concatenate([idx[:2], r.choice(n, 126, replace=False)])]
    queries = list(r.choice(n, 6, replace=False)) + [int(idx[0])]
    for q in queries:
        hq = halves + [np.concatenate([[q], r.choice(n, 127, replace=False)])]
        for half in hq:
          for cands in (half[:8], half[8:16], half[-8:]):
            cands = [int(c) for c in cands]
            for shift in (-1.0, 0.0, 1.0):
                v_mmas = []
                for c in cands:
                    exact = float(np.dot(V[q].astype(np.float64), V[c].astype(np.float64)))
                    v_mmas.append(F(exact + shift * c_split * float(vn[q]) * float(vn[c])))
                for kpick in (0, 1):
                    g = group_hi(q, half, cands, data, v_mmas, kpick)
                    for c, v in zip(cands, v_mmas):
                        if c == q:
                            continue  # the query itself: phase 1 marks it +inf (never rejected, see below)
                        for pick in (0, 1, 2):
                            _, bhi = epilogue_rho_bounds(q, c, data, v, pick, raw=True)
                            assert g >= bhi, (q, cands, c, float(g), float(bhi))
                    if q in cands:  # the group holding the query can never be rejected
                        isq = data[3][q]
                        assert float(g) >= (1.0 - 2e-6) / float(isq)


def _kv_variants(q, c, data, pick):
    """The kernel value of pair_kv2 (screen_sweep_kernel) for one pair, float32 operation by
    operation, in every form the compiler may produce: each entry is (kv, exact product
    whose rounding is kv, d2, a, e^-a), with the Matern polynomial's a^2/3 term fused into
    its add or not."""
    Vf, xs, vn, isp, xmax, xmax_max, var, kt, m, d = data
    d2 = F(0.0)
    for a_ in range(d):
        t = F(xs[c, a_] + F(-xs[q, a_]))
        d2 = fma32(t, t, d2)
    if kt == 0:
        e = expf_band(F(F(-0.5) * d2))[pick]
        return [(F(F(var) * e), np.float64(var) * np.float64(e), d2, F(0.0), F(0.0))]
    a = F(F(2.2360679775) * F(np.sqrt(d2)))
    ea = expf_band(F(-a))[pick]
    out = []
    for fuse_poly in (False, True):
        a2 = F(a * a)
        one_a = F(F(1.0) + a)
        poly = F(np.float64(a2) * np.float64(F(0.33333334)) + np.float64(one_a)) if fuse_poly \
            else F(one_a + F(a2 * F(0.33333334)))
        vp = F(F(var) * poly)
        out.append((F(vp * ea), np.float64(vp) * np.float64(ea), d2, a, ea))
    return out


def _dif_variants(kv, prod, v):
    """kv - s with the product kept (rounded kv) or fused into the add (one rounding)."""
    return [F(kv + F(-v)), F(prod - np.float64(v))]


def _phase1_bhi(q, c, data, kv, dif, d2, a, ea):
    Vf, xs, vn, isp, xmax, xmax_max, var, kt, m, d = data
    u2 = 1.0 / 65536.0
    err_coef = F(3.1 * u2 + (3.0 * m / 16.0 + 17.0) * 2.0 ** -22)
    err_c = F(err_coef * vn[c])
    dd = F(d)
    ced2 = F(F(dd + F(2.0)) * F(5.97e-8))
    A = F(F(2.4e-7) * F(xmax[q] + xmax_max))
    ale = F(F(ced2 + F(F(F(0.5) * A) * dd)) * F(1.00001))
    bee = F(F(F(0.5) * A) * F(1.00001))
    alk = F(F(F(F(6e-8) + F(F(0.5) * ced2)) + F(F(F(0.25) * A) * dd)) * F(1.00001))
    bek = F(F(F(1e-6) + F(F(0.25) * A)) * F(1.00001))
    if kt == 0:
        ek = F(kv * fma32(alk, d2, bek))
    else:
        ed2 = fma32(ale, d2, bee)
        t1 = F(kv * F(F(1e-6) + F(F(2.4e-7) * a)))
        t2 = F(F(F(F(var) * F(F(F(0.8334) * ed2) + F(F(F(1e-7) * a) * a))) * F(F(1.0) + a)) * ea)
        ek = F(t1 + t2)
    R = F(abs(dif))
    e = F(fma32(vn[q], err_c, ek) + fma32(R, F(1.2e-7), F(1e-30)))
    return F(F(R + e) * isp[c])


@pytest.mark.parametrize("n,d,m,kt,ls", [
    (1500, 8, 64, 0, 2.0),   # RBF, precision-workload-like
    (1500, 3, 64, 1, 1.0),   # Matern 5/2
    (1200, 3, 128, 0, 0.7),  # RBF, short lengthscale
    (1200, 5, 96, 1, 2.0),   # Matern, D = 5
])
def test_second_tier_bounds_every_pair(n, d, m, kt, ls):
    """The sweep's second group tier (per-pair kernel values, screen_sweep_kernel) never
    rejects a group holding a pair that phase 1 would keep or heap: with 2.4e-7 kv added to
    each |kv - s|, its bound is >= phase 1's survivor bound bhi of every pair, whichever of
    the two tiers has the kernel value's last multiply (and the Matern polynomial's) fused
    into the following add, for tensor-core dots anywhere in the certified band and __expf
    at either end of its band; groups of near points (where the tier decides), random groups
    and groups with tiny-p rows."""
    X, V, p, idx, data = _case(n, d, m, kt, ls, seed=n + d + m + 7)
    xs, vn, isp = data[1], data[2], data[3]
    u2 = 1.0 / 65536.0
    err_coef = F(3.1 * u2 + (3.0 * m / 16.0 + 17.0) * 2.0 ** -22)
    c_split = 3.1 * u2 + (3.0 * m / 16.0 + 17.0) * 2.0 ** -22
    r = np.random.default_rng(29)
    order = np.lexsort(tuple(xs[:, a] for a in range(d)))
    groups = [order[s:s + 8] for s in r.choice(n - 8, 8, replace=False)]
    groups += [r.choice(n, 8, replace=False) for _ in range(3)]
    groups += [np.concatenate([idx[:2], r.choice(n, 6, replace=False)])]
    queries = [int(g[3]) for g in groups[:5]] + [int(idx[0])]  # members of near groups, an inducing row
    checked = 0
    for q in queries:
        ekmax = _query_consts(q, data)
        for g in groups:
            cands = [int(c) for c in g if int(c) != q]
            err_max = max(F(err_coef * vn[c]) for c in cands)
            isc_max = max(isp[c] for c in cands)
            for shift in (-1.0, 0.0, 1.0):
                vs = {c: F(float(np.dot(V[q].astype(np.float64), V[c].astype(np.float64)))
                           + shift * c_split * float(vn[q]) * float(vn[c])) for c in cands}
                for pick in (0, 1, 2):
                    kvs = {c: _kv_variants(q, c, data, pick) for c in cands}
                    # tier 2 in each compiled form (the same form for every pair of the group)
                    n_forms = len(kvs[cands[0]]) * 2
                    for form in range(n_forms):
                        rc = F(0.0)
                        for c in cands:
                            kv, prod, _, _, _ = kvs[c][form // 2]
                            dif = _dif_variants(kv, prod, vs[c])[form % 2]
                            rc = max(rc, fma32(kv, F(2.4e-7), F(abs(dif))))
                        inner = F(F(F(rc * F(1.0 + 3e-7)) + F(vn[q] * err_max)) + F(ekmax + F(1e-30)))
                        gc = F(F(inner * isc_max) * F(1.0 + 1e-6))
                        for c in cands:
                            for kv, prod, d2, a, ea in kvs[c]:
                                for dif in _dif_variants(kv, prod, vs[c]):
                                    bhi = _phase1_bhi(q, c, data, kv, dif, d2, a, ea)
                                    assert gc >= bhi, (q, c, form, pick, float(gc), float(bhi))
                                    checked += 1
    assert checked > 1000
