"""The LBVH's box growth rests on one rounding bound of the reference's sphere
test (src/renderer/cpu.rs:34-62, the expanded quadratic in f32): a hit can be
reported only when the ray's line passes within

    rho^2 <= r^2 (1 + 2^-20) + 2^-19 (|o| + |c|)^2

of the centre.  numpy's float32 arithmetic rounds every operation exactly as
the reference does (no contraction), so the bound is checked here on rays
aimed to graze spheres just outside their radius, with origins and centres
far from the world origin, where the rounding is largest."""
import numpy as np

U = 2.0 ** -24


def _hits(o, d, c, r):
    """The reference's hit decision (disc >= 0 and a root >= 0), per ray."""
    f = np.float32
    dot = lambda x, y: (x[:, 0] * y[:, 0] + x[:, 1] * y[:, 1]) + x[:, 2] * y[:, 2]
    a = dot(d, d)
    k = dot(o, d) - dot(d, c)
    cc = ((dot(o, o) - f(2) * dot(o, c)) + dot(c, c)) - r * r
    disc = k * k - a * cc
    with np.errstate(invalid="ignore"):
        sq = np.sqrt(disc)
        t1 = (-k - sq) / a
        t2 = (-k + sq) / a
    return (disc >= 0) & ((t1 >= 0) | (t2 >= 0))


def _grazing(rng, n, scale_o, scale_c, r_lo, r_hi, slack):
    """Rays whose exact line misses a sphere by rho = r + slack * |o|+|c| * 2^-10."""
    c = rng.uniform(-scale_c, scale_c, (n, 3))
    r = np.exp(rng.uniform(np.log(r_lo), np.log(r_hi), n))
    o = c + rng.normal(size=(n, 3)) * scale_o
    # direction towards a point at distance rho from c, perpendicular to (c - o)
    w = c - o
    p = np.cross(w, rng.normal(size=(n, 3)))
    p /= np.linalg.norm(p, axis=1, keepdims=True)
    s = np.linalg.norm(o, axis=1) + np.linalg.norm(c, axis=1)
    rho = r + slack * rng.uniform(0, 1, n) * s * 2.0 ** -10
    d = (c + p * rho[:, None]) - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d *= rng.uniform(0.5, 2.0, (n, 1))  # scattered directions are not unit length
    f = np.float32
    return o.astype(f), d.astype(f), c.astype(f), r.astype(f)


def _rho2_and_s(o, d, c, r):
    o, d, c, r = (x.astype(np.float64) for x in (o, d, c, r))
    w = o - c
    proj = (w * d).sum(1) / (d * d).sum(1)
    rho2 = ((w - proj[:, None] * d) ** 2).sum(1)
    s = np.linalg.norm(o, axis=1) + np.linalg.norm(c, axis=1)
    return rho2, s, r


def test_sphere_hits_stay_inside_the_grown_radius():
    rng = np.random.default_rng(11)
    worst = 0.0
    n_hits = 0
    for scale_o, scale_c, r_lo, r_hi in [(40, 30, 1e-3, 0.2), (2000, 30, 1e-2, 1.0), (5, 1e4, 1e-3, 10.0),
                                         (1e5, 1e5, 1e-2, 1.0), (0.5, 1e3, 1e-4, 1e-2)]:
        for slack in (0.25, 1.0, 4.0):
            o, d, c, r = _grazing(rng, 200_000, scale_o, scale_c, r_lo, r_hi, slack)
            hit = _hits(o, d, c, r)
            rho2, s, rr = _rho2_and_s(o, d, c, r)
            miss = rho2 > rr * rr
            spurious = hit & miss
            n_hits += int(spurious.sum())
            bound = rr * rr * (1 + 2.0 ** -20) + 2.0 ** -19 * s * s
            assert np.all(rho2[hit] <= bound[hit]), "a hit outside the grown radius"
            if spurious.any():
                worst = max(worst, float(((rho2 - rr * rr) / (U * s * s))[spurious].max()))
    # rounding does produce hits on rays that miss, and they stay well inside
    # the 32 u S^2 the leaf boxes allow (21 u S^2 is the first-order bound)
    assert n_hits > 100
    assert worst < 21.0
