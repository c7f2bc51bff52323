"""Seeded synthetic initial conditions (G = 1) for tests and the benchmark.

The reference generates its scenes with Go's math/rand/v2 PCG (internal/scene/scene.go), whose
exact streams are not reproduced here; these generators follow the same published recipes with
numpy's PCG64, and every consumer (the CUDA library and the CPU oracle) reads the identical
arrays, so parity never depends on the generator.

  plummer(n)            Aarseth-Henon-Wielen (1974) Plummer sphere, truncated at 20a
                        (the method of scene.go:380-404)
  test_disk(n)          the reference's bh_test.go galaxy(n): thin exponential disk of Salpeter
                        masses around a central hole, plus a second hole (bh_test.go:54-63)
  galaxy(n)             exponential Toomre-Q disk (40 %), Hernquist bulge (10 %) and an NFW halo
                        (50 %, 4x the disk particle mass) truncated at 10 r_s; halo and bulge
                        velocities from Eddington's formula in the total potential
  merger(n)             two galaxy(n/2) on a parabolic orbit
  far_cluster()         the clumpy cluster plus probe of bh_test.go:294-307
  forest(nsys)          independent Plummer or galaxy systems of log-uniform sizes, one state
  adjoint_problem(n)    Plummer sphere with lognormal masses and rotated, noisy target positions
                        (the differentiable workload)
"""
from __future__ import annotations

import numpy as np

STAR, BLACK_HOLE, DARK_MATTER = 0, 1, 2


def _state(pos, vel, mass, kind=None):
    n = len(mass)
    return dict(px=np.ascontiguousarray(pos[:, 0], np.float64), py=np.ascontiguousarray(pos[:, 1], np.float64),
                pz=np.ascontiguousarray(pos[:, 2], np.float64), vx=np.ascontiguousarray(vel[:, 0], np.float64),
                vy=np.ascontiguousarray(vel[:, 1], np.float64), vz=np.ascontiguousarray(vel[:, 2], np.float64),
                ax=np.zeros(n), ay=np.zeros(n), az=np.zeros(n), mass=np.ascontiguousarray(mass, np.float64),
                kind=np.zeros(n, np.uint8) if kind is None else np.ascontiguousarray(kind, np.uint8),
                alive=np.ones(n, np.uint8))


def _directions(rng, n):
    z = 2 * rng.random(n) - 1
    phi = 2 * np.pi * rng.random(n)
    r = np.sqrt(1 - z * z)
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)


def plummer(n: int, seed: int = 0, mass: float = 1.0, a: float = 1.0, rcut: float = 20.0, float32: bool = True):
    """Equal-mass Plummer sphere (AHW 1974), mass fraction inside rcut*a only."""
    rng = np.random.default_rng(seed)
    fmax = rcut ** 3 / (1 + rcut ** 2) ** 1.5
    x = rng.random(n) * fmax
    x = np.maximum(x, 1e-12)
    r = a / np.sqrt(x ** (-2.0 / 3.0) - 1)
    q = np.empty(n)
    todo = np.arange(n)
    while len(todo):
        qq = rng.random(len(todo))
        ok = 0.1 * rng.random(len(todo)) < qq * qq * (1 - qq * qq) ** 3.5
        q[todo[ok]] = qq[ok]
        todo = todo[~ok]
    ve = np.sqrt(2 * mass) * (r * r + a * a) ** -0.25
    pos = _directions(rng, n) * r[:, None]
    vel = _directions(rng, n) * (q * ve)[:, None]
    pos -= pos.mean(axis=0)
    vel -= vel.mean(axis=0)
    if float32:  # positions and velocities stored as float32
        pos = pos.astype(np.float32).astype(np.float64)
        vel = vel.astype(np.float32).astype(np.float64)
    return _state(pos, vel, np.full(n, mass / n))


def _salpeter(rng, n, total, lo=0.1, hi=10.0, alpha=2.35):
    k = 1 - alpha
    a, b = lo ** k, hi ** k
    m = (a + (b - a) * rng.random(n)) ** (1 / k)
    return m * (total / m.sum())


def test_disk(n: int, seed: int = 1, holes: bool = True):
    """Disk of n stars (total mass 1, Salpeter masses), scale radius 0.8 in [0.15, 4], thickness
    0.03, dispersion 0.12 of circular speed; central hole of mass 2 and a hole of 0.5 at (1.5, 0.3)
    when holes is set. Softening 0.06 in the reference's test."""
    rng = np.random.default_rng(seed)
    masses = _salpeter(rng, n, 1.0)
    r = np.empty(n)
    todo = np.arange(n)
    while len(todo):
        rr = -0.8 * np.log(rng.random(len(todo)) * rng.random(len(todo)))
        ok = (rr >= 0.15) & (rr <= 4)
        r[todo[ok]] = rr[ok]
        todo = todo[~ok]
    r.sort()
    phi = rng.random(n) * 2 * np.pi
    z = rng.normal(size=n) * 0.03
    eps2 = 0.06 ** 2
    enclosed = 2.0 + np.cumsum(masses)
    r2 = r * r + z * z + eps2
    vc = np.sqrt(enclosed * r * r / (r2 * np.sqrt(r2)))
    disp = 0.12 * vc
    pos = np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)
    vel = np.stack([-vc * np.sin(phi) + rng.normal(size=n) * disp, vc * np.cos(phi) + rng.normal(size=n) * disp,
                    rng.normal(size=n) * disp], axis=1)
    kind = np.zeros(n, np.uint8)
    if holes:
        pos = np.vstack([[0, 0, 0], pos, [1.5, 0.3, 0]])
        vel = np.vstack([[0, 0, 0], vel, [0, 0, 0]])
        masses = np.concatenate([[2.0], masses, [0.5]])
        kind = np.concatenate([[BLACK_HOLE], kind, [BLACK_HOLE]]).astype(np.uint8)
    return _state(pos, vel, masses, kind)


def far_cluster(seed: int = 5):
    """A clumpy cluster of radius ~1 around (10, 3, -2) and a light probe at the origin."""
    rng = np.random.default_rng(seed)
    pos = [np.zeros(3)]
    m = [1e-9]
    for i in range(400):
        off = np.array([0.5 * (i % 2), 0.3 * (i % 3), 0.0])
        pos.append(np.array([10 + rng.normal() * 0.4, 3 + rng.normal() * 0.2, -2 + rng.normal() * 0.3]) + off)
        m.append(0.5 + rng.random())
    pos = np.array(pos)
    return _state(pos, np.zeros_like(pos), np.array(m))


# ---------------------------------------------------------------- galaxy model


class _Spherical:
    """Enclosed-mass profiles of the galaxy model, spherically averaged."""

    def __init__(self, m_disk, r_d, m_bulge, a_b, m_halo, r_s, r_t):
        self.m_disk, self.r_d, self.m_bulge, self.a_b = m_disk, r_d, m_bulge, a_b
        self.m_halo, self.r_s, self.r_t = m_halo, r_s, r_t
        self._mu_t = np.log1p(r_t / r_s) - (r_t / r_s) / (1 + r_t / r_s)
        self._hb = (r_t + a_b) ** 2 / r_t ** 2  # Hernquist truncated at r_t holds m_bulge

    def halo_mass(self, r):
        x = np.minimum(r, self.r_t) / self.r_s
        return self.m_halo * (np.log1p(x) - x / (1 + x)) / self._mu_t

    def halo_rho(self, r):
        x = r / self.r_s
        rho0 = self.m_halo / (4 * np.pi * self.r_s ** 3 * self._mu_t)
        return np.where(r <= self.r_t, rho0 / (x * (1 + x) ** 2), 0.0)

    def bulge_mass(self, r):
        r = np.minimum(r, self.r_t)
        return self.m_bulge * self._hb * r * r / (r + self.a_b) ** 2

    def bulge_rho(self, r):
        mt = self.m_bulge * self._hb
        return np.where(r <= self.r_t, mt * self.a_b / (2 * np.pi * r * (r + self.a_b) ** 3), 0.0)

    def disk_mass(self, r):
        y = r / self.r_d
        return self.m_disk * (1 - (1 + y) * np.exp(-y))

    def mass(self, r):
        return self.halo_mass(r) + self.bulge_mass(r) + self.disk_mass(r)


def _eddington_sampler(model: _Spherical, rho_fn, r_t):
    """Tabulates f(E) of a component of density rho_fn in the model's total potential
    (Eddington's formula, Binney & Tremaine eq. 4.46b) and returns (psi(r), sample(r, rng))."""
    r = np.logspace(np.log10(r_t) - 6, np.log10(r_t), 4000)
    m = model.mass(r)
    dpsi_dr = -m / r ** 2
    # psi(r) = int_r^rt M/r'^2 dr' (zero at the truncation radius)
    seg = 0.5 * (m[1:] / r[1:] ** 2 + m[:-1] / r[:-1] ** 2) * np.diff(r)
    psi = np.concatenate([np.cumsum(seg[::-1])[::-1], [0.0]])
    rho = rho_fn(r)
    drho_dr = np.gradient(rho, r)
    drho_dpsi = drho_dr / dpsi_dr  # >= 0
    # as functions of psi (increasing order)
    ps, dr = psi[::-1], drho_dpsi[::-1]
    e_grid = np.linspace(0, psi[0], 1200)[1:]
    u = np.linspace(0, 1, 400)
    # g(E) = int_0^E drho/dpsi dpsi / sqrt(E - psi) = int_0^sqrt(E) 2 drho/dpsi(E - w^2) dw
    g = np.empty_like(e_grid)
    for i, e in enumerate(e_grid):
        w = u * np.sqrt(e)
        vals = 2 * np.interp(e - w * w, ps, dr)
        g[i] = np.trapezoid(vals, w)
    f = np.gradient(g, e_grid) / (np.sqrt(8) * np.pi ** 2)
    f = np.maximum(f, 0.0)

    def psi_at(rr):
        return np.interp(rr, r, psi)

    def sample(rr, rng):
        p = psi_at(rr)
        vmax = np.sqrt(2 * np.maximum(p, 0))
        out = np.zeros(len(rr))
        # per-particle bound of v^2 f(psi - v^2/2) on a coarse grid, with margin
        t = np.linspace(0, 1, 33)[None, :]
        vv = vmax[:, None] * t
        dens = vv ** 2 * np.interp(p[:, None] - vv ** 2 / 2, e_grid, f, left=0.0)
        bound = dens.max(axis=1) * 1.3 + 1e-300
        todo = np.arange(len(rr))
        for _ in range(200):
            if not len(todo):
                break
            v = vmax[todo] * rng.random(len(todo))
            d = v * v * np.interp(p[todo] - v * v / 2, e_grid, f, left=0.0)
            ok = rng.random(len(todo)) * bound[todo] < d
            out[todo[ok]] = v[ok]
            todo = todo[~ok]
        out[todo] = 0.5 * vmax[todo]
        return out

    return psi_at, sample


def _rotate(vecs, incl, orient=0.0):
    ci, si = np.cos(incl), np.sin(incl)
    rx = np.array([[1, 0, 0], [0, ci, -si], [0, si, ci]])
    co, so = np.cos(orient), np.sin(orient)
    rz = np.array([[co, -so, 0], [so, co, 0], [0, 0, 1]])
    return vecs @ (rz @ rx).T


def galaxy(n: int, seed: int = 0, q_toomre: float = 1.5, incl: float = 0.0, orient: float = 0.0,
           r_d: float = 1.0, z0: float = 0.1, a_b: float = 0.2, r_s: float = 5.0, c: float = 10.0,
           float32: bool = True):
    """Disk (40 % of particles, mass 1), bulge (10 %, same particle mass) and NFW halo (50 %,
    four times the disk particle mass, r_s = 5, truncated at c * r_s)."""
    rng = np.random.default_rng(seed)
    n_d = int(round(0.4 * n))
    n_b = int(round(0.1 * n))
    n_h = n - n_d - n_b
    m_p = 1.0 / n_d
    m_disk, m_bulge, m_halo = n_d * m_p, n_b * m_p, n_h * 4 * m_p
    r_t = c * r_s
    model = _Spherical(m_disk, r_d, m_bulge, a_b, m_halo, r_s, r_t)

    # halo positions: invert M(<r) numerically
    rg = np.logspace(-5, np.log10(r_t), 20000)
    frac = model.halo_mass(rg) / m_halo
    r_h = np.interp(rng.random(n_h), frac, rg)
    _, halo_v = _eddington_sampler(model, model.halo_rho, r_t)
    v_h = halo_v(r_h, rng)
    pos_h = _directions(rng, n_h) * r_h[:, None]
    vel_h = _directions(rng, n_h) * v_h[:, None]

    # bulge: Hernquist truncated at r_t, M(<r) ~ r^2/(r+a)^2
    s = np.sqrt(rng.random(n_b) / model._hb)
    r_b = a_b * s / (1 - s)
    _, bulge_v = _eddington_sampler(model, model.bulge_rho, r_t)
    v_b = bulge_v(r_b, rng)
    pos_b = _directions(rng, n_b) * r_b[:, None]
    vel_b = _directions(rng, n_b) * v_b[:, None]

    # disk: R ~ Gamma(2, r_d) below 10 r_d, z ~ sech^2(z/z0); Toomre-Q dispersions (Hernquist 1993)
    R = np.empty(n_d)
    todo = np.arange(n_d)
    while len(todo):
        rr = rng.gamma(2.0, r_d, len(todo))
        ok = rr < 10 * r_d
        R[todo[ok]] = rr[ok]
        todo = todo[~ok]
    z = z0 * np.arctanh(np.clip(2 * rng.random(n_d) - 1, -0.999999, 0.999999))
    phi = rng.random(n_d) * 2 * np.pi
    Rs = np.maximum(R, 1e-3)
    vc2 = model.mass(Rs) / Rs
    h = 1e-3
    om2 = lambda x: model.mass(x) / x ** 3
    dom2 = (om2(Rs + h) - om2(np.maximum(Rs - h, 1e-4))) / (2 * h)
    kappa2 = np.maximum(Rs * dom2 + 4 * om2(Rs), 1e-12)
    sigma_surf = m_disk / (2 * np.pi * r_d ** 2) * np.exp(-Rs / r_d)
    sig_r = q_toomre * 3.36 * sigma_surf / np.sqrt(kappa2)
    sig_p = sig_r * np.sqrt(kappa2) / (2 * np.sqrt(om2(Rs)))
    sig_z = np.sqrt(np.pi * sigma_surf * z0)
    vphi2 = vc2 + sig_r ** 2 * (1 - kappa2 / (4 * om2(Rs)) - 2 * Rs / r_d)
    vphi = np.sqrt(np.maximum(vphi2, 0.0)) + rng.normal(size=n_d) * sig_p
    vr = rng.normal(size=n_d) * sig_r
    vz = rng.normal(size=n_d) * sig_z
    cp, sp = np.cos(phi), np.sin(phi)
    pos_d = np.stack([R * cp, R * sp, z], axis=1)
    vel_d = np.stack([vr * cp - vphi * sp, vr * sp + vphi * cp, vz], axis=1)

    pos = np.vstack([pos_d, pos_b, pos_h])
    vel = np.vstack([vel_d, vel_b, vel_h])
    mass = np.concatenate([np.full(n_d, m_p), np.full(n_b, m_p), np.full(n_h, 4 * m_p)])
    kind = np.concatenate([np.zeros(n_d + n_b, np.uint8), np.full(n_h, DARK_MATTER, np.uint8)])
    pos = _rotate(pos, incl, orient)
    vel = _rotate(vel, incl, orient)
    mtot = mass.sum()
    pos -= (mass[:, None] * pos).sum(axis=0) / mtot
    vel -= (mass[:, None] * vel).sum(axis=0) / mtot
    if float32:
        pos = pos.astype(np.float32).astype(np.float64)
        vel = vel.astype(np.float32).astype(np.float64)
    return _state(pos, vel, mass, kind)


def merger(n: int, seed: int = 0, pericentre: float = 5.0, separation: float = 40.0,
           incl1: float = np.radians(30.0), incl2: float = np.radians(60.0)):
    """Two equal galaxy(n/2) models on a parabolic orbit (pericentre, starting separation)."""
    n1 = n // 2
    g1 = galaxy(n1, seed=seed, incl=incl1)
    g2 = galaxy(n - n1, seed=seed + 1, incl=incl2, orient=np.radians(45.0))
    m1, m2 = g1["mass"].sum(), g2["mass"].sum()
    mt = m1 + m2
    # relative parabolic orbit: r = 2q / (1 + cos f); v^2 = 2 G M / r
    cosf = 2 * pericentre / separation - 1
    f = -np.arccos(np.clip(cosf, -1, 1))  # approaching
    r = separation
    rel_pos = np.array([r * np.cos(f), r * np.sin(f), 0.0])
    # velocity of a parabola: v_r = sqrt(GM/p) e sin f, v_t = sqrt(GM/p)(1 + e cos f), p = 2q, e = 1
    p = 2 * pericentre
    k = np.sqrt(mt / p)
    vr, vt = k * np.sin(f), k * (1 + np.cos(f))
    rel_vel = np.array([vr * np.cos(f) - vt * np.sin(f), vr * np.sin(f) + vt * np.cos(f), 0.0])
    off1, off2 = -m2 / mt, m1 / mt
    out = {}
    for key in ("px", "py", "pz", "vx", "vy", "vz"):
        ax = "xyz".index(key[1])
        d = rel_pos[ax] if key[0] == "p" else rel_vel[ax]
        out[key] = np.concatenate([g1[key] + off1 * d, g2[key] + off2 * d])
    for key in ("ax", "ay", "az", "mass", "kind", "alive"):
        out[key] = np.concatenate([g1[key], g2[key]])
    return out


def forest(nsys: int = 64, seed: int = 0, nmin: int = 2048, nmax: int = 65536, scale=(0.5, 2.0)):
    """nsys independent systems concatenated into one state: each N log-uniform in [nmin, nmax],
    scale radius uniform in `scale`, a Plummer sphere or a disk+bulge+halo galaxy by its seed.
    Returns (state, offsets) with offsets[s] the first body of system s."""
    rng = np.random.default_rng(seed)
    parts, offsets = [], [0]
    for q in range(nsys):
        n = int(round(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
        a = rng.uniform(*scale)
        if rng.random() < 0.5:
            s = plummer(n, seed=seed * 1000 + q, a=a)
        else:
            s = galaxy(max(n, 16), seed=seed * 1000 + q, r_d=a, z0=0.1 * a, a_b=0.2 * a, r_s=5 * a)
        parts.append(s)
        offsets.append(offsets[-1] + len(s["px"]))
    out = {k: np.concatenate([p[k] for p in parts]) for k in parts[0]}
    return out, np.array(offsets, np.int64)


def adjoint_problem(n: int, seed: int = 0, sigma: float = 0.3, angle_deg: float = 30.0, noise: float = 0.01):
    """A Plummer sphere (positions and velocities as plummer(n, seed), in FP64) with masses
    lognormal(0, sigma) normalised to a total of 1, and targets = initial positions rotated by
    angle_deg about z plus N(0, noise^2) per coordinate. Returns (state, targets n x 3)."""
    s = plummer(n, seed=seed, float32=False)
    rng = np.random.default_rng(seed + 7919)
    m = np.exp(rng.normal(0.0, sigma, n))
    s["mass"] = m / m.sum()
    t = np.radians(angle_deg)
    c, si = np.cos(t), np.sin(t)
    x0 = np.stack([s["px"], s["py"], s["pz"]], 1)
    rot = np.array([[c, -si, 0.0], [si, c, 0.0], [0.0, 0.0, 1.0]])
    targets = x0 @ rot.T + rng.normal(0.0, noise, (n, 3))
    return s, targets
