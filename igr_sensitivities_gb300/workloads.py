"""Host-side problem set-up: initial conditions and time steps.

Mirrors the builders of IGR_adjoints_2d/initial_conditions.jl and
IGR_adjoints_1d/initial_conditions.jl that the tests use, plus the seeded
Gaussian-pulse family the benchmark workloads are drawn from (ambient gas at
rest, rho = 1, p = 0.1 + sum_k A_k exp(-|x - c_k|^2 / w^2), E = p/(gamma-1),
the form of build_sedov_blast_ic!, initial_conditions.jl:136-150). Seeds feed
a SplitMix64 generator so that the same seed gives the same instance on every
machine.
"""
import numpy as np

MASK64 = (1 << 64) - 1


class SplitMix64:
    def __init__(self, seed):
        self.s = seed & MASK64

    def next_u64(self):
        self.s = (self.s + 0x9E3779B97F4A7C15) & MASK64
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
        return z ^ (z >> 31)

    def uniform(self, lo=0.0, hi=1.0):
        return lo + (hi - lo) * ((self.next_u64() >> 11) * (1.0 / (1 << 53)))


def seed_for(config_id, instance):
    return 0x16150000 + config_id * (1 << 20) + instance


def pulse_ic_2d(mesh, gamma, amps, centers, width, p_bg=0.1):
    """rho = 1, u = 0, p = p_bg + sum A exp(-r^2/width^2) (periodic images ignored)."""
    x, y = mesh.x, mesh.y
    p = np.full(x.shape, p_bg)
    for A, (xc, yc) in zip(amps, centers):
        p = p + A * np.exp(-((x - xc) ** 2 + (y - yc) ** 2) / width ** 2)
    rho = np.ones(x.shape)
    z = np.zeros(x.shape)
    return (np.asfortranarray(z), np.asfortranarray(z.copy()), np.asfortranarray(rho), np.asfortranarray(p / (gamma - 1)))


def seeded_pulses_2d(mesh, gamma, seed, n_pulses=3, width=0.03, amp=(1.0, 10.0), lo=0.2, hi=0.8):
    rng = SplitMix64(seed)
    amps = [rng.uniform(*amp) for _ in range(n_pulses)]
    centers = [(rng.uniform(lo, hi), rng.uniform(lo, hi)) for _ in range(n_pulses)]
    return pulse_ic_2d(mesh, gamma, amps, centers, width)


def seeded_window(seed):
    """Square window (x0, y0, side) for the window_rho2 objective."""
    rng = SplitMix64(seed ^ 0x5DEECE66D)
    side = rng.uniform(0.2, 0.4)
    return (rng.uniform(0.0, 0.6), rng.uniform(0.0, 0.6), side)


def taylor_green_ic(mesh, gamma, A):
    """build_taylor_green_ic!, IGR_adjoints_2d/initial_conditions.jl:105-121."""
    cx = 2 * np.pi * mesh.x / mesh.Lx
    cy = 2 * np.pi * mesh.y / mesh.Ly
    ux = A * np.sin(cx) * np.cos(cy)
    uy = -A * np.cos(cx) * np.sin(cy)
    rho = np.ones(mesh.x.shape)
    return (np.asfortranarray(rho * ux), np.asfortranarray(rho * uy), np.asfortranarray(rho),
            np.asfortranarray(1.0 / (gamma - 1) + 0.5 * rho * (ux ** 2 + uy ** 2)))


def max_wavespeed_2d(mux, muy, rho, E, gamma):
    P = (gamma - 1) * (E - (mux ** 2 + muy ** 2) / (2 * rho))
    c = np.sqrt(gamma * P / rho)
    return float(max(np.max(np.abs(mux / rho) + c), np.max(np.abs(muy / rho) + c)))


def cfl_dt_2d(mesh, p, q, gamma, cfl):
    """dt = CFL min(dx, dy) / ((2p+1) max wavespeed) (IGR_adjoints_2d/tests/run_euler_test.jl:100-106)."""
    return cfl * min(mesh.dx, mesh.dy) / ((2 * p + 1) * max_wavespeed_2d(*q, gamma))


# ----------------------------------------------------------------------------- 1D
def pulse_ic_1d(mesh, gamma, amps, centers, width, p_bg=0.1):
    """1D pressure pulses at rest: rho = 1, u = 0, p = p_bg + sum A exp(-(x-c)^2/width^2);
    returns (mu, rho, E) shaped (n_p, N_e)."""
    x = mesh.x
    p = np.full(x.shape, p_bg)
    for A, c in zip(amps, centers):
        p = p + A * np.exp(-((x - c) ** 2) / width ** 2)
    return (np.asfortranarray(np.zeros(x.shape)), np.asfortranarray(np.ones(x.shape)),
            np.asfortranarray(p / (gamma - 1)))


def seeded_pulses_1d(mesh, gamma, seed, n_pulses=2, width=0.02, amp=(1.0, 10.0), lo=0.2, hi=0.8):
    rng = SplitMix64(seed)
    amps = [rng.uniform(*amp) for _ in range(n_pulses)]
    centers = [rng.uniform(lo, hi) for _ in range(n_pulses)]
    return pulse_ic_1d(mesh, gamma, amps, centers, width)


def seeded_interval(seed):
    """Interval [a, b] for the interval_rho objective."""
    rng = SplitMix64(seed ^ 0x2545F4914F6CDD1D)
    a = rng.uniform(0.1, 0.6)
    return (a, a + rng.uniform(0.1, 0.3))


def max_wavespeed_1d(mu, rho, E, gamma):
    P = (gamma - 1) * (E - mu ** 2 / (2 * rho))
    return float(np.max(np.abs(mu / rho) + np.sqrt(gamma * P / rho)))


def cfl_dt_1d(mesh, p, q, gamma, cfl):
    """dt = CFL dx / ((2p+1) max wavespeed), the 1D form of the tests' CFL rule."""
    return cfl * mesh.dx / ((2 * p + 1) * max_wavespeed_1d(*q, gamma))


def oseen_pair_pulse_2d(mesh, gamma, seed, a_core=0.05, circ=(0.5, 1.0), amp=(1.0, 10.0), pulse_width=0.05,
                        n_tab=4000):
    """Counter-rotating Oseen vortex pair plus one Gaussian pressure pulse
    (the family of build_oseen_pair_blast_ic!, IGR_adjoints_2d/initial_conditions.jl:175-232):
    v_theta = G/(2 pi r) (1 - exp(-r^2/a^2)) summed over 3x3 periodic images,
    homentropic radial equilibrium through the enthalpy defect
    D(r) = (G/2pi)^2 int_r^inf (1 - e^{-s^2/a^2})^2 / s^3 ds (tabulated,
    composed additively for the pair), ambient p = rho = 1. The pair (zero net
    circulation, as the doubly periodic box requires) is centred at a seeded
    point with separation 0.2; the pulse sits at a seeded point.

    The circulation is drawn as a fraction U[circ] of the strongest vortex
    that keeps the core enthalpy defect D(0) = (G/2pi)^2 ln2 / a^2 at or below
    a quarter of the ambient enthalpy gamma/(gamma-1): a literal circulation of
    order one would drive the core pressure negative at ambient p = 1.
    """
    rng = SplitMix64(seed)
    L = mesh.Lx
    g_max = 2 * np.pi * a_core * np.sqrt(0.25 * gamma / (gamma - 1) / np.log(2.0))
    G = rng.uniform(*circ) * g_max
    xc, yc = rng.uniform(0.3, 0.7), rng.uniform(0.3, 0.7)
    A = rng.uniform(*amp)
    bx, by = rng.uniform(0.2, 0.8), rng.uniform(0.2, 0.8)
    centers = ((xc, yc + 0.1, +1.0), (xc, yc - 0.1, -1.0))
    r_max = 2.0 * L
    r_tab = np.linspace(0.0, r_max, n_tab)
    with np.errstate(divide="ignore", invalid="ignore"):
        f = np.where(r_tab < 1e-12, 0.0, (1.0 - np.exp(-r_tab ** 2 / a_core ** 2)) ** 2 / r_tab ** 3)
    seg = 0.5 * (f[:-1] + f[1:]) * np.diff(r_tab)
    D_tab = np.zeros(n_tab)
    D_tab[:-1] = (G / (2 * np.pi)) ** 2 * np.cumsum(seg[::-1])[::-1]

    def defect(r):
        t = np.clip(r / r_max * (n_tab - 1), 0, n_tab - 1 - 1e-12)
        i = np.floor(t).astype(int)
        w = t - i
        return np.where(r >= r_max, 0.0, (1 - w) * D_tab[i] + w * D_tab[np.minimum(i + 1, n_tab - 1)])

    x, y = mesh.x, mesh.y
    ux, uy = np.zeros(x.shape), np.zeros(x.shape)
    h = np.full(x.shape, gamma / (gamma - 1))
    for cx, cy, sgn in centers:
        for sx in (-1, 0, 1):
            for sy in (-1, 0, 1):
                dx, dy = x - (cx + sx * L), y - (cy + sy * L)
                r2 = dx ** 2 + dy ** 2
                with np.errstate(divide="ignore", invalid="ignore"):
                    v = np.where(r2 < 1e-24, 0.0, sgn * G / (2 * np.pi * r2) * (1.0 - np.exp(-r2 / a_core ** 2)))
                ux += -v * dy
                uy += v * dx
        dx, dy = x - cx, y - cy
        dx -= L * np.round(dx / L)
        dy -= L * np.round(dy / L)
        h = h - defect(np.sqrt(dx ** 2 + dy ** 2))
    p_v = ((gamma - 1) * h / gamma) ** (gamma / (gamma - 1))
    rho = p_v ** (1.0 / gamma)
    p = p_v + A * np.exp(-((x - bx) ** 2 + (y - by) ** 2) / pulse_width ** 2)
    E = p / (gamma - 1) + 0.5 * rho * (ux ** 2 + uy ** 2)
    return tuple(np.asfortranarray(a) for a in (rho * ux, rho * uy, rho, E))
