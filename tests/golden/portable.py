"""Catalogs that come out bit-identical on every IEEE-754 machine, for the fixtures whose
inputs are too large to store (200K-point catalogs with the benchmark configurations'
shapes and binnings).

The stream is splitmix64 (Steele, Lea and Flood, "Fast splittable pseudorandom number
generators", OOPSLA 2014) in numpy uint64 arithmetic, which wraps the same way everywhere.
Every float is made from it with correctly rounded operations only (+, -, *, /, sqrt), never
with a library transcendental (whose last bit may differ between x86 and Arm libm), so the
reference run that made a fixture and a test on another machine see the same bits.

  * uniform(n): (u >> 11) * 2^-53, exact doubles in [0, 1).
  * approx_normal(n, sigma): the Irwin-Hall sum of 4 uniforms, centred and scaled to the
    given standard deviation (a smooth stand-in for the Gaussian shears of the benchmark
    configurations; exact arithmetic).
  * directions on a spherical cap from z uniform in [cos r, 1] and a rejection-sampled unit
    vector in the plane (no sine or cosine), rotated by an exact 120-degree turn about the x
    axis so the cap sits at dec = -30 deg, away from the pole.
"""
import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


class Stream:
    def __init__(self, seed):
        self.state = np.uint64(seed & 0xFFFFFFFFFFFFFFFF)

    def u64(self, n):
        with np.errstate(over="ignore"):
            k = np.arange(1, n + 1, dtype=np.uint64)
            z = self.state + k * np.uint64(0x9E3779B97F4A7C15)
            self.state = z[-1] if n else self.state
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            z = z ^ (z >> np.uint64(31))
        return z

    def uniform(self, n):
        return (self.u64(n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)

    def approx_normal(self, n, sigma):
        u = self.uniform(4 * n).reshape(4, n)
        s = ((u[0] + u[1]) + (u[2] + u[3])) - 2.0
        return s * (sigma * np.sqrt(3.0))   # Irwin-Hall(4) has variance 4/12


def _shear(st, n, sigma):
    g1 = st.approx_normal(n, sigma)
    g2 = st.approx_normal(n, sigma)
    gsq = g1 * g1 + g2 * g2
    shrink = np.where(gsq > 0.81, 0.9 / np.sqrt(np.maximum(gsq, 1e-300)), 1.0)
    return g1 * shrink, g2 * shrink


def flat_catalog(seed, n, L, sigma=0.2):
    """x, y ~ U[0, L]; g1, g2 ~ approx N(0, sigma) with |g| < 0.9; k ~ approx N(0, 0.02);
    w ~ U[0.5, 1.5]."""
    st = Stream(seed)
    x = st.uniform(n) * L
    y = st.uniform(n) * L
    g1, g2 = _shear(st, n, sigma)
    k = st.approx_normal(n, 0.02)
    w = st.uniform(n) + 0.5
    return dict(x=x, y=y, z=None, g1=g1, g2=g2, k=k, w=w)


def cap_catalog(seed, n, cos_r, sigma=0.25):
    """Unit vectors uniform on the cap of angular radius r (given as cos r) centred at
    dec = -30 deg; shears, k and w as flat_catalog."""
    st = Stream(seed)
    z0 = cos_r + st.uniform(n) * (1.0 - cos_r)
    a = np.empty(n)
    b = np.empty(n)
    filled = 0
    while filled < n:
        m = 2 * (n - filled) + 64
        ua = st.uniform(m) * 2.0 - 1.0
        ub = st.uniform(m) * 2.0 - 1.0
        q = ua * ua + ub * ub
        ok = (q > 1e-6) & (q <= 1.0)
        take = min(int(ok.sum()), n - filled)
        a[filled:filled + take] = ua[ok][:take]
        b[filled:filled + take] = ub[ok][:take]
        filled += take
    rn = np.sqrt(a * a + b * b)
    s = np.sqrt((1.0 - z0) * (1.0 + z0))
    x0 = s * (a / rn)
    y0 = s * (b / rn)
    # Rotation by 120 deg about x: the pole goes to dec = -30 deg.
    c, sn = -0.5, np.sqrt(0.75)
    x = x0
    y = c * y0 - sn * z0
    z = sn * y0 + c * z0
    g1, g2 = _shear(st, n, sigma)
    k = st.approx_normal(n, 0.02)
    w = st.uniform(n) + 0.5
    return dict(x=x.copy(), y=y.copy(), z=z.copy(), g1=g1, g2=g2, k=k, w=w)


# cos of the angular radius of a 1000 deg^2 cap: area = 2 pi (1 - cos r) sr.
COS_R_1000DEG2 = 1.0 - 1000.0 * ((np.pi / 180.0) * (np.pi / 180.0)) / (2.0 * np.pi)
