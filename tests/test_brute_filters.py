"""The brute-force kernels' pass 1 on the guarded fast path is a conservative
filter, not the reference's test: it may keep a sphere or cube the reference
misses, never drop one it hits (src/renderer/cpu.rs:34-62 spheres, 64-98
cubes; pass 2 then decides every kept object with the reference's own
arithmetic).

Its float operations are restated here in numpy float32, each FMA as
float32(float64(a) * float64(b) + float64(c)): the product is exact in
float64, so the result is the single-rounded FMA except in rare
double-rounding ties, where it is one ulp away; the filter's margin is more
than three times its first-order rounding bound.  The reference's decision
(disc >= 0 and a root >= 0, non-fused float32) is the one the oracle
computes.  Inputs: rays grazing spheres just outside and inside their
radius, rays leaving a sphere's surface (the self-intersection case whose
roots straddle 0), far origins and centres, huge and tiny radii; rays aimed
at cube edges and corners, starting on cube faces and inside cubes."""
import numpy as np

F = np.float32


def _fma(a, b, c):
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(F)


def _dot(x, y):
    return (x[:, 0] * y[:, 0] + x[:, 1] * y[:, 1]) + x[:, 2] * y[:, 2]


def _reference_hits(o, d, c, r):
    a = _dot(d, d)
    k = _dot(o, d) - _dot(d, c)
    cc = ((_dot(o, o) - F(2) * _dot(o, c)) + _dot(c, c)) - r * r
    disc = k * k - a * cc
    with np.errstate(invalid="ignore"):
        sq = np.sqrt(disc)
        t1 = (-k - sq) / a
        t2 = (-k + sq) / a
    return (disc >= 0) & ((t1 >= 0) | (t2 >= 0))


def _filter_s(c, rr):
    """rdc_flatten.hpp sphere_filter_s: c.c - q rounded down, q = r^2 + 2^-16 (2 c.c + r^2) + 2^-70."""
    cd = c.astype(np.float64)
    cc = (cd * cd).sum(1)
    q = (rr.astype(np.float64) + np.ldexp(2.0 * cc + rr, -16) + 2.0 ** -70) * (1.0 + 2.0 ** -40)
    v = cc - q
    sd = v - np.abs(v) * 2.0 ** -45 - np.ldexp(cc + q, -50)
    f = sd.astype(F)
    high = f.astype(np.float64) > sd
    f[high] = np.nextafter(f[high], F(-np.inf))
    return f


def _filter_keeps(o, d, c, r):
    """sphere_candidates<true> (rdc_device.cuh), one sphere per row."""
    rr = r * r
    s_ = _filter_s(c, rr)
    a = _dot(d, d)
    oo = _dot(o, o)
    od = _dot(o, d)
    P = (a * F(2.0 ** -15)) * oo
    b = _fma(-d[:, 2], c[:, 2], _fma(-d[:, 1], c[:, 1], _fma(-d[:, 0], c[:, 0], od)))
    m2o = F(-2) * o
    e = _fma(m2o[:, 2], c[:, 2], _fma(m2o[:, 1], c[:, 1], _fma(m2o[:, 0], c[:, 0], oo + s_)))
    disc = _fma(b, b, _fma(-a, e, P))
    return ~np.signbit(disc)


def _unit(v):
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def _grazing(rng, n, scale_o, scale_c, r_lo, r_hi, rel):
    """Rays whose line passes at rho = r (1 + rel * U(-1, 1)) from the centre."""
    c = rng.uniform(-scale_c, scale_c, (n, 3))
    r = np.exp(rng.uniform(np.log(r_lo), np.log(r_hi), n))
    o = c + _unit(rng.normal(size=(n, 3))) * (r * rng.uniform(1.5, 50.0, n))[:, None] * scale_o
    w = c - o
    p = _unit(np.cross(w, rng.normal(size=(n, 3))))
    rho = r * (1 + rel * rng.uniform(-1, 1, n))
    d = (c + p * rho[:, None]) - o
    d = _unit(d) * rng.uniform(0.25, 3.0, (n, 1))
    if rng.uniform() < 0.5:
        d = -d  # the sphere behind the origin
    return o.astype(F), d.astype(F), c.astype(F), r.astype(F)


def _leaving(rng, n, scale_c, r_lo, r_hi):
    """Rays starting on (the float rounding of) a sphere's surface, any direction."""
    c = rng.uniform(-scale_c, scale_c, (n, 3))
    r = np.exp(rng.uniform(np.log(r_lo), np.log(r_hi), n))
    o = c + _unit(rng.normal(size=(n, 3))) * r[:, None]
    d = _unit(rng.normal(size=(n, 3))) * rng.uniform(0.25, 3.0, (n, 1))
    return o.astype(F), d.astype(F), c.astype(F), r.astype(F)


CASES = [(1.0, 30, 1e-3, 0.5), (4.0, 1000, 1e-2, 2.0), (1.0, 5, 1e-4, 1e-2), (0.2, 2e4, 1.0, 500.0),
         (1.0, 1e3, 900.0, 1100.0), (1.0, 1e5, 1e-2, 1.0)]


def _check(o, d, c, r):
    hit = _reference_hits(o, d, c, r)
    keep = _filter_keeps(o, d, c, r)
    dropped = hit & ~keep
    assert not dropped.any(), f"filter drops {int(dropped.sum())} reference hits, first at {np.argmax(dropped)}"
    return hit, keep


def test_filter_never_drops_a_grazing_hit():
    rng = np.random.default_rng(5)
    n_hit = 0
    for scale_o, scale_c, r_lo, r_hi in CASES:
        for rel in (1e-3, 1e-5, 1e-7):
            o, d, c, r = _grazing(rng, 100_000, scale_o, scale_c, r_lo, r_hi, rel)
            hit, _ = _check(o, d, c, r)
            n_hit += int(hit.sum())
    assert n_hit > 100_000  # (these rays' lines all pass inside the margin band: every one is kept)


def test_filter_never_drops_a_hit_from_the_surface():
    rng = np.random.default_rng(6)
    n_hit = 0
    for _, scale_c, r_lo, r_hi in CASES:
        o, d, c, r = _leaving(rng, 200_000, scale_c, r_lo, r_hi)
        hit, _ = _check(o, d, c, r)
        n_hit += int(hit.sum())
    assert n_hit > 10_000  # rounding and inward rays do hit the sphere they leave


def test_filter_culls_clear_misses():
    rng = np.random.default_rng(7)
    n = 100_000
    c = rng.uniform(-20, 20, (n, 3)).astype(F)
    r = rng.uniform(0.1, 1.0, n).astype(F)
    o = (c + _unit(rng.normal(size=(n, 3))) * (r * 3)[:, None] + rng.uniform(-1, 1, (n, 3))).astype(F)
    d = _unit(rng.normal(size=(n, 3))).astype(F)
    hit, keep = _check(o, d, c, r)
    w = (o - c).astype(np.float64)
    dd = d.astype(np.float64)
    b = (w * dd).sum(1)
    ww = (w * w).sum(1)
    rho2 = ww - b * b / (dd * dd).sum(1)
    r2 = r.astype(np.float64) ** 2
    # the margin widens r^2 by 2^-16 (2 |o|^2 + 2 |c|^2 + r^2)
    band = 2.0 ** -16 * (2 * (o.astype(np.float64) ** 2).sum(1) + 2 * (c.astype(np.float64) ** 2).sum(1) + r2)
    far_miss = rho2 > r2 + 1.1 * band
    assert far_miss.sum() > n // 2
    assert not keep[far_miss].any()
    assert keep[hit].all()
    # spheres wholly behind the origin are kept when their line passes through
    # them (pass 2 rejects them): the filter tests the line, not the half-line
    behind_through = (b > 0) & (ww > 1.5 * r2) & (rho2 < 0.9 * r2)
    assert behind_through.sum() > 100
    assert keep[behind_through].all() and not hit[behind_through].any()


# ---- cubes ---------------------------------------------------------------


def _reference_cube_t(o, d, lo, hi):
    """hit_cube (cpu.rs:64-98) in float32: t of a hit, NaN for None."""
    with np.errstate(divide="ignore", invalid="ignore"):
        t0 = (lo - o) / d
        t1 = (hi - o) / d
    tmin = np.max(np.minimum(t0, t1), axis=1)
    tmax = np.min(np.maximum(t0, t1), axis=1)
    hit = ~(tmax < 0) & ~(tmin > tmax)
    t = np.where(tmin < 0, tmax, tmin)
    return np.where(hit, t, np.nan).astype(F)


def _cube_run_bound(c, h):
    """rdc_flatten.hpp cube_run_bound over the given cubes."""
    R = (np.sqrt((c.astype(np.float64) ** 2).sum(1)) + np.abs(h.astype(np.float64)) * np.sqrt(3.0)).max() * 1.0001
    f = F(R)
    return np.nextafter(f, F(np.inf)) if float(f) < R else f


def _cube_filter_keeps(o, d, lo, hi, R):
    """cube_filter_ray + cube_candidates (rdc_device.cuh), one cube per row."""
    inv = (F(1) / d).astype(F)
    ol1 = (np.abs(o[:, 0]) + np.abs(o[:, 1])) + np.abs(o[:, 2])
    m = F(2.0 ** -20) * (ol1 + F(2) * R) + F(1e-30)
    oa = (o + m[:, None]) * inv
    ob = (o - m[:, None]) * inv
    pos = inv >= 0
    sn = np.where(pos, oa, ob)
    sf = np.where(pos, ob, oa)
    nf = F(2.0 ** -120) - sf
    near = np.where(pos, lo, hi)
    far = np.where(pos, hi, lo)
    e = _fma(near, inv, -sn)
    x = _fma(far, inv, nf)
    entry = e.max(axis=1)
    exit_ = x.min(axis=1)
    s = np.signbit
    return ~(s(exit_ - entry) | s(exit_))


def _cubes(rng, n, scale_c, h_lo, h_hi):
    c = rng.uniform(-scale_c, scale_c, (n, 3)).astype(F)
    h = (np.exp(rng.uniform(np.log(h_lo), np.log(h_hi), n)).astype(F) * F(2)) * F(0.5)
    return c, h, (c - h[:, None]).astype(F), (c + h[:, None]).astype(F)


def _cube_rays(rng, c, h, mode):
    n = len(c)
    hd = h.astype(np.float64)[:, None]
    cd = c.astype(np.float64)
    if mode == "edge":
        # aim at a point on an edge or corner of the box, perturbed by a few ulp-scales
        target = cd + hd * np.sign(rng.normal(size=(n, 3))) * (1 + rng.uniform(-1e-6, 1e-6, (n, 3)))
        keep_axis = rng.integers(0, 3, n)
        target[np.arange(n), keep_axis] = cd[np.arange(n), keep_axis] + hd[:, 0] * rng.uniform(-1, 1, n)
        o = cd + _unit(rng.normal(size=(n, 3))) * hd * rng.uniform(2, 40, (n, 1))
        d = target - o
    elif mode == "face":
        # start on (the rounding of) a face, any direction
        o = cd + hd * rng.uniform(-1, 1, (n, 3))
        ax = rng.integers(0, 3, n)
        o[np.arange(n), ax] = cd[np.arange(n), ax] + hd[:, 0] * np.sign(rng.normal(size=n))
        d = rng.normal(size=(n, 3))
    else:  # inside
        o = cd + hd * rng.uniform(-0.999, 0.999, (n, 3))
        d = rng.normal(size=(n, 3))
    d = _unit(d) * rng.uniform(0.25, 3.0, (n, 1))
    small = np.abs(d) < 2.0 ** -30  # the fast path's range guard
    d[small] = 2.0 ** -30
    return o.astype(F), d.astype(F)


def test_cube_filter_never_drops_a_hit():
    rng = np.random.default_rng(8)
    n_hit = 0
    for scale_c, h_lo, h_hi in [(30, 0.05, 2.0), (1e4, 1.0, 50.0), (2, 1e-3, 1e-2), (1e5, 1e-2, 1.0)]:
        for mode in ("edge", "face", "inside"):
            c, h, lo, hi = _cubes(rng, 100_000, scale_c, h_lo, h_hi)
            o, d = _cube_rays(rng, c, h, mode)
            t = _reference_cube_t(o, d, lo, hi)
            hit = ~np.isnan(t)
            R = _cube_run_bound(c, h)
            keep = _cube_filter_keeps(o, d, lo, hi, R)
            assert not (hit & ~keep).any(), f"{mode}: a reference hit dropped"
            n_hit += int(hit.sum())
    assert n_hit > 200_000


def test_cube_filter_culls_clear_misses():
    rng = np.random.default_rng(9)
    c, h, lo, hi = _cubes(rng, 100_000, 20, 0.1, 1.0)
    o = (c + _unit(rng.normal(size=(len(c), 3))) * (h * 4)[:, None]).astype(F)
    d = _unit(rng.normal(size=(len(c), 3))).astype(F)
    t = _reference_cube_t(o, d, lo, hi)
    keep = _cube_filter_keeps(o, d, lo, hi, _cube_run_bound(c, h))
    hit = ~np.isnan(t)
    assert not (hit & ~keep).any()
    # the box grown by about 2^-20 (|o| + 2R) keeps hardly anything the cube misses
    assert (keep & ~hit).sum() < 0.01 * (~hit).sum()
    assert (~keep).sum() > 0.5 * len(c)
