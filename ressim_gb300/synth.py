"""Seeded synthetic black-oil Newton systems (input generator for benchmarks and size-independent tests).

The reference produces its Jacobians with its full black-oil simulator (engine/src/simulator.cpp:2500-3033),
which is not part of this solver. For the large configurations (60x220x85 SPE10-model-2-sized grid, the
64-realisation 40x40x10 ensemble, the serving stream) this module builds Jacobians of the same structure
directly, in the style of the reference's own synthetic test matrices (``testMatrix``,
app/src/gpu_compute.cpp:720-750; ``makeBlockLaplace``, tests/run_tests.cpp:3694-3724) but with the physics
shape of the assembled system:

* cells on a Cartesian grid (natural ordering, i fastest), optional ACTNUM mask, active cells renumbered in
  natural order; 7-point TPFA connections with harmonic-mean transmissibilities;
* unknowns per cell (p, Sw, Sg), equations (water, oil, gas) in surface volumes, rows scaled by dt / PV as the
  reference scales them (engine/src/simulator.cpp:3303-3310), upstream-weighted Corey mobilities with their
  saturation derivatives, accumulation derivatives (the true-IMPES ``acc`` blocks);
* log-normal correlated permeability (Gaussian moving-average filter per layer, as ``generateRock``,
  engine/src/tools.cpp:195-245), optional seeded binary channels, porosity phi = 0.05 + 0.02 ln k;
* wells with one BHP unknown each (rate-controlled producers and water injectors); the well rows are
  eliminated exactly (S = Acc - Acw Dww^-1 Awc, engine/src/bsr.cpp:733-840), which adds the fill blocks that
  couple all perforated cells of a well;
* a manufactured solution x_true and b = S x_true, so every solve can be checked against a known answer.

Nothing here is on the timed path: it only produces inputs.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.ndimage import gaussian_filter1d

from .bsr import BSR, NewtonSystem, ScalarCSR

NB = 3
SWC, SOR, SGC = 0.2, 0.2, 0.05
MU = (0.5, 1.5, 0.02)          # cp: water, oil, gas
BF = (1.0 / 1.02, 1.0 / 1.25, 1.0 / 0.006)   # inverse formation volume factors (surface / reservoir)
RS = 0.45                      # dissolved gas-oil ratio
COMP = (3e-6, 1.2e-5, 4e-4)    # phase compressibilities (1/psi)
CROCK = 4e-6


def correlated_normal(shape, corr, rng):
    """Unit-variance Gaussian field, independent per layer, filtered in y then x (corr in cells)."""
    nz, ny, nx = shape
    w = rng.standard_normal(shape)
    f = w
    if corr[1] > 0:
        f = gaussian_filter1d(f, sigma=0.5 * corr[1], axis=1, mode="reflect")
    if corr[0] > 0:
        f = gaussian_filter1d(f, sigma=0.5 * corr[0], axis=2, mode="reflect")
    if len(corr) > 2 and corr[2] > 1:
        f = gaussian_filter1d(f, sigma=0.5 * corr[2], axis=0, mode="reflect")
    s = f.reshape(nz, -1).std(axis=1)
    s[s == 0] = 1.0
    return f / s[:, None, None]


def channel_mask(nx, ny, nz, layers, width, rng, n_channels=None):
    """Seeded sinuous binary channels along y, ``width`` cells wide, in the given layers."""
    m = np.zeros((nz, ny, nx), dtype=bool)
    jj = np.arange(ny)[:, None]
    ii = np.arange(nx)[None, :]
    for k in layers:
        nc = n_channels if n_channels is not None else max(1, nx // 20)
        for _ in range(nc):
            x0 = rng.uniform(0, nx)
            amp = rng.uniform(2, max(3.0, nx / 6))
            lam = rng.uniform(ny / 3, ny)
            ph = rng.uniform(0, 2 * math.pi)
            xc = x0 + amp * np.sin(2 * math.pi * jj / lam + ph)
            m[k] |= np.abs(ii - xc) < 0.5 * width
    return m


def _corey(sw, sg):
    """Mobilities (per phase) and their derivatives w.r.t. (Sw, Sg)."""
    den = 1.0 - SWC - SOR
    se = np.clip((sw - SWC) / den, 0.0, 1.0)
    dse = np.where((sw > SWC) & (sw < 1 - SOR), 1.0 / den, 0.0)
    krw = 0.6 * se**2
    dkrw = 1.2 * se * dse
    sgn = np.clip((sg - SGC) / (1.0 - SWC - SGC), 0.0, 1.0)
    dsgn = np.where(sg > SGC, 1.0 / (1.0 - SWC - SGC), 0.0)
    krg = 0.8 * sgn**2
    dkrg = 1.6 * sgn * dsgn
    so_n = np.clip((1.0 - sw - sg - SOR) / (1.0 - SWC - SOR), 0.0, 1.0)
    dso = np.where((so_n > 0) & (so_n < 1), -1.0 / (1.0 - SWC - SOR), 0.0)
    kro = so_n**2
    dkro = 2.0 * so_n * dso   # same derivative w.r.t. Sw and Sg
    lw, lo, lg = krw / MU[0], kro / MU[1], krg / MU[2]
    # surface-volume mobilities of the three equations: water, oil, gas (free + dissolved)
    lam = np.stack([BF[0] * lw, BF[1] * lo, BF[2] * lg + RS * BF[1] * lo], axis=-1)
    dlam_sw = np.stack([BF[0] * dkrw / MU[0], BF[1] * dkro / MU[1], RS * BF[1] * dkro / MU[1]], axis=-1)
    dlam_sg = np.stack([np.zeros_like(sw), BF[1] * dkro / MU[1], BF[2] * dkrg / MU[2] + RS * BF[1] * dkro / MU[1]], axis=-1)
    lt = lw + lo + lg
    dlt_sw = dkrw / MU[0] + dkro / MU[1]
    dlt_sg = dkro / MU[1] + dkrg / MU[2]
    return lam, dlam_sw, dlam_sg, lt, dlt_sw, dlt_sg


def make_system(nx, ny, nz, *, sigma=1.0, corr=(5, 5, 1), seed=0, dx=100.0, dy=100.0, dz=20.0, kmean=100.0,
                actnum_fraction=0.0, channels=None, wells="corners+center", n_wells=None, dt=1.0, porosity=None,
                with_full=False, xtrue_seed=None, front_radius=0.5, gravity_head=False, p_noise=5.0) -> NewtonSystem:
    """Build one Schur-reduced black-oil Newton system.

    channels: None or (first_layer, last_layer, width, multiplier) (layers zero-based inclusive).
    wells: "corners+center" (central water injector + 4 corner producers, all layers, as tools/gen_bigcase.py:44-52),
           "diagonal" (injector at (0,0), producer at (nx-1,ny-1), all layers), or "random" (n_wells seeded columns).
    gravity_head: upwind and flux by the flow potential p - 0.45 psi/ft x depth (the hydrostatic gradient of the
           initial pressure), so that vertical connections carry only the well-driven part of the pressure field, as in
           a simulator's state at equilibrium; False: by the pressure difference alone.
    p_noise: standard deviation (psi) of the per-cell pressure perturbation.
    """
    rng = np.random.default_rng(seed)
    shape = (nz, ny, nx)
    z = correlated_normal(shape, corr, rng)
    lnk = math.log(kmean) + sigma * z
    if channels is not None:
        k0, k1, width, mult = channels
        cm = channel_mask(nx, ny, nz, range(k0, min(k1, nz - 1) + 1), width, rng)
        lnk = np.where(cm, lnk + math.log(mult), lnk)
    k = np.exp(lnk)
    phi = np.clip(0.05 + 0.02 * lnk if porosity is None else np.full(shape, porosity), 0.01, 0.45)
    active = np.ones(shape, dtype=bool)
    if actnum_fraction > 0:
        f = correlated_normal(shape, (6, 6, 2), rng)
        thr = np.quantile(f, actnum_fraction)
        active = f > thr
    ncell = nx * ny * nz
    act_flat = active.reshape(-1)
    idx = np.full(ncell, -1, dtype=np.int64)
    na = int(act_flat.sum())
    idx[act_flat] = np.arange(na)
    kf = k.reshape(-1)[act_flat]
    phif = phi.reshape(-1)[act_flat]
    kk_, jj_, ii_ = np.unravel_index(np.nonzero(act_flat)[0], shape)
    depth = (kk_ + 0.5) * dz

    # ---- state: pressure and saturation fields around the wells
    ci, cj = (nx - 1) / 2.0, (ny - 1) / 2.0
    well_cols = []
    if wells == "corners+center":
        well_cols = [("INJ", int(round(ci)), int(round(cj)), "inj")] + [
            ("P%d" % (q + 1), i, j, "prod") for q, (i, j) in enumerate([(0, 0), (nx - 1, 0), (0, ny - 1), (nx - 1, ny - 1)])]
    elif wells == "diagonal":
        well_cols = [("INJ", 0, 0, "inj"), ("PROD", nx - 1, ny - 1, "prod")]
    elif wells == "random":
        nwr = n_wells if n_wells is not None else 2
        for q in range(nwr):
            well_cols.append(("W%d" % q, int(rng.integers(0, nx)), int(rng.integers(0, ny)), "inj" if q % 3 == 0 else "prod"))
    L = 0.35 * math.hypot(nx * dx, ny * dy)
    p = 4000.0 + 0.45 * depth
    front = np.zeros(na)
    for (_, wi, wj, kind) in well_cols:
        r = np.hypot((ii_ - wi) * dx, (jj_ - wj) * dy) + 0.5 * dx
        if kind == "inj":
            p = p + 600.0 * np.exp(-r / L)
            front = np.maximum(front, 1.0 / (1.0 + np.exp((r - front_radius * L) / (0.1 * L))))
        else:
            p = p - 400.0 * np.exp(-r / L)
    p = p + p_noise * rng.standard_normal(na)
    sw = SWC + (1 - SWC - SOR) * front * (0.8 + 0.2 * rng.random(na))
    sw = np.clip(sw + 0.02 * rng.random(na), SWC, 1 - SOR - 1e-3)
    sg = np.where(kk_ < max(1, nz // 4), 0.1 * rng.random(na) * (1.0 - front), 0.0)
    sg = np.clip(sg, 0.0, 1.0 - sw - SOR - 1e-3)
    lam, dlsw, dlsg, lt, dltsw, dltsg = _corey(sw, sg)

    pv = phif * dx * dy * dz / 5.615        # reservoir barrels
    scale = dt / pv                          # row scaling dt / PV

    # ---- accumulation derivatives per unit pore volume (rows: water, oil, gas; cols: p, Sw, Sg)
    so = 1.0 - sw - sg
    acc = np.zeros((na, 3, 3))
    acc[:, 0, 0] = BF[0] * sw * (CROCK + COMP[0])
    acc[:, 0, 1] = BF[0]
    acc[:, 1, 0] = BF[1] * so * (CROCK + COMP[1])
    acc[:, 1, 1] = -BF[1]
    acc[:, 1, 2] = -BF[1]
    acc[:, 2, 0] = BF[2] * sg * (CROCK + COMP[2]) + RS * BF[1] * so * (CROCK + COMP[1]) + 1e-4 * BF[1] * so
    acc[:, 2, 1] = -RS * BF[1]
    acc[:, 2, 2] = BF[2] - RS * BF[1]

    # ---- connections (i < j in active numbering): +x, +y, +z neighbours
    conns = []
    for (di, dj, dk, area, dist) in ((1, 0, 0, dy * dz, dx), (0, 1, 0, dx * dz, dy), (0, 0, 1, dx * dy, dz)):
        m = np.ones(shape, dtype=bool)
        if di:
            m[:, :, -1] = False
        if dj:
            m[:, -1, :] = False
        if dk:
            m[-1, :, :] = False
        src = np.nonzero(m.reshape(-1))[0]
        dst = src + di + dj * nx + dk * nx * ny
        a, b_ = idx[src], idx[dst]
        ok = (a >= 0) & (b_ >= 0)
        a, b_ = a[ok], b_[ok]
        kz = 0.1 if dk else 1.0
        kh = 2.0 / (1.0 / (kz * kf[a]) + 1.0 / (kz * kf[b_]))
        T = 0.001127 * kh * area / dist
        conns.append((a, b_, T))
    ca = np.concatenate([c[0] for c in conns])
    cb = np.concatenate([c[1] for c in conns])
    cT = np.concatenate([c[2] for c in conns])
    dpc = p[cb] - p[ca]                                   # flow from a to b when dpc < 0
    if gravity_head:
        dpc = dpc - 0.45 * (depth[cb] - depth[ca])
    up = np.where(dpc < 0, ca, cb)
    lam_u = lam[up]                                        # (nc, 3)
    dsw_u = dlsw[up]
    dsg_u = dlsg[up]
    up_is_a = up == ca

    # flux into a from b: F = T lam_u (p_b - p_a); residual R_a -= F, R_b += F (rows scaled by dt/PV)
    # d R_a / d x:   p_a: +T lam, p_b: -T lam, S_u: -T dp dlam
    # d R_b / d x:   p_a: -T lam, p_b: +T lam, S_u: +T dp dlam
    nconn = ca.size
    blk_aa = np.zeros((nconn, 3, 3)); blk_ab = np.zeros((nconn, 3, 3))
    blk_ba = np.zeros((nconn, 3, 3)); blk_bb = np.zeros((nconn, 3, 3))
    Tl = cT[:, None] * lam_u
    blk_aa[:, :, 0] += Tl; blk_ab[:, :, 0] -= Tl
    blk_ba[:, :, 0] -= Tl; blk_bb[:, :, 0] += Tl
    gs = -(cT * dpc)[:, None]
    dS = np.stack([dsw_u, dsg_u], axis=-1) * gs[:, :, None]          # (nc, 3 eq, 2 sat)
    ua = up_is_a[:, None, None]
    blk_aa[:, :, 1:] += np.where(ua, dS, 0.0)
    blk_ab[:, :, 1:] += np.where(ua, 0.0, dS)
    blk_ba[:, :, 1:] -= np.where(ua, dS, 0.0)
    blk_bb[:, :, 1:] -= np.where(ua, 0.0, dS)
    sa = scale[ca][:, None, None]
    sb = scale[cb][:, None, None]
    diag = acc.copy()
    np.add.at(diag, ca, sa * blk_aa)
    np.add.at(diag, cb, sb * blk_bb)

    # ---- wells: one BHP unknown each; perforations in every active layer of the column
    wrow_cells, wcw, wwc, Dw, wnames = [], [], [], [], []
    for (name, wi, wj, kind) in well_cols:
        cells = idx[(np.arange(nz) * ny + wj) * nx + wi]
        cells = cells[cells >= 0]
        if cells.size == 0:
            continue
        WI = 2.0 * 0.001127 * kf[cells] * dz / math.log(0.2 * dx / 0.25)
        pw = p[cells].mean() + (300.0 if kind == "inj" else -300.0)
        if kind == "inj":
            # water injection with total mobility; only the water equation gets the source
            c_cw = np.zeros((cells.size, 3))
            c_cw[:, 0] = -scale[cells] * WI * lt[cells] * BF[0]
            dpp = np.zeros((cells.size, 3, 3))
            dpp[:, 0, 0] = scale[cells] * WI * lt[cells] * BF[0]
            wc = np.zeros((cells.size, 3))
            wc[:, 0] = -WI * lt[cells]
            wc[:, 1] = WI * (pw - p[cells]) * dltsw[cells]
            wc[:, 2] = WI * (pw - p[cells]) * dltsg[cells]
            D = float(np.sum(WI * lt[cells]))
        else:
            c_cw = -scale[cells][:, None] * WI[:, None] * lam[cells]
            dpp = np.zeros((cells.size, 3, 3))
            dpp[:, :, 0] = scale[cells][:, None] * WI[:, None] * lam[cells]
            dd = (p[cells] - pw)
            dpp[:, :, 1] = scale[cells][:, None] * (WI * dd)[:, None] * dlsw[cells]
            dpp[:, :, 2] = scale[cells][:, None] * (WI * dd)[:, None] * dlsg[cells]
            wc = np.zeros((cells.size, 3))
            wc[:, 0] = WI * lt[cells]
            wc[:, 1] = WI * dd * dltsw[cells]
            wc[:, 2] = WI * dd * dltsg[cells]
            D = -float(np.sum(WI * lt[cells]))
        np.add.at(diag, cells, dpp)
        wrow_cells.append(cells); wcw.append(c_cw); wwc.append(wc); Dw.append(D); wnames.append(name)
    nw = len(Dw)

    # ---- assemble the cell block matrix + Schur fill, merged and sorted per row
    rows = [np.arange(na), ca, cb]
    cols = [np.arange(na), cb, ca]
    vals = [diag, sa * blk_ab, sb * blk_ba]
    for w in range(nw):
        cells = wrow_cells[w]
        m = cells.size
        ri = np.repeat(cells, m)
        cj = np.tile(cells, m)
        fill = -(wcw[w][:, None, :, None] * wwc[w][None, :, None, :]) / Dw[w]     # (m, m, 3 eq, 3 col)
        rows.append(ri); cols.append(cj); vals.append(fill.reshape(m * m, 3, 3))
    R = np.concatenate(rows).astype(np.int64)
    Cc = np.concatenate(cols).astype(np.int64)
    V = np.concatenate(vals, axis=0)
    key = R * na + Cc
    order = np.argsort(key, kind="stable")
    key_s = key[order]
    uniq, start = np.unique(key_s, return_index=True)
    Vs = np.add.reduceat(V[order], start, axis=0)
    ur = (uniq // na).astype(np.int32)
    uc = (uniq % na).astype(np.int32)
    rowPtr = np.zeros(na + 1, dtype=np.int32)
    np.add.at(rowPtr, ur + 1, 1)
    rowPtr = np.cumsum(rowPtr, dtype=np.int64).astype(np.int32)
    A = BSR(na, NB, rowPtr, uc, Vs.reshape(-1))

    # ---- manufactured solution and right-hand side b = S x_true
    rng2 = np.random.default_rng(seed + 7919 if xtrue_seed is None else xtrue_seed)
    xt = np.empty((na, 3))
    xt[:, 0] = 20.0 * np.sin(0.05 * ii_ + 0.07 * jj_) * np.cos(0.3 * kk_) + rng2.standard_normal(na)
    xt[:, 1] = 0.01 * rng2.standard_normal(na)
    xt[:, 2] = 0.005 * rng2.standard_normal(na)
    xt = xt.reshape(-1)
    b = bsr_matvec_host(A, xt)

    full = None
    full_b = None
    if with_full:
        full, full_b = _full_jacobian(A, na, nw, diag, ca, cb, sa * blk_ab, sb * blk_ba, wrow_cells, wcw, wwc, Dw, xt, rng2)
    meta = dict(nx=nx, ny=ny, nz=nz, sigma=sigma, seed=seed, wells=wnames, dt=dt, active=na)
    return NewtonSystem(A, b, acc=acc.reshape(-1), full=full, full_b=full_b, na=na, nv=3, nw=nw, x_true=xt, meta=meta)


def bsr_matvec_host(A: BSR, x: np.ndarray) -> np.ndarray:
    """Host matvec used only to manufacture right-hand sides for generated inputs."""
    blk = A.blocks()
    xv = x.reshape(A.n, A.nb)
    contrib = np.einsum("kij,kj->ki", blk, xv[A.col])
    rows = np.repeat(np.arange(A.n), np.diff(A.rowPtr))
    y = np.zeros((A.n, A.nb))
    np.add.at(y, rows, contrib)
    return y.reshape(-1)


def _full_jacobian(A, na, nw, diag, ca, cb, bab, bba, wcells, wcw, wwc, Dw, xt, rng):
    """Scalar CSR with well rows (cells first, then one BHP row per well), values before the Schur step, and its
    right-hand side for a manufactured (cells, BHP) solution."""
    nc = na * 3
    ent_r, ent_c, ent_v = [], [], []

    def add_blocks(bi, bj, blocks):
        e = np.arange(3)
        r = (bi[:, None, None] * 3 + e[None, :, None]).repeat(3, axis=2)
        c = (bj[:, None, None] * 3 + e[None, None, :]).repeat(3, axis=1)
        ent_r.append(r.reshape(-1)); ent_c.append(c.reshape(-1)); ent_v.append(blocks.reshape(-1))

    add_blocks(np.arange(na), np.arange(na), diag)
    add_blocks(ca, cb, bab)
    add_blocks(cb, ca, bba)
    for w in range(nw):
        cells = wcells[w]
        for e in range(3):
            ent_r.append(cells * 3 + e); ent_c.append(np.full(cells.size, nc + w)); ent_v.append(wcw[w][:, e])
        for e in range(3):
            ent_r.append(np.full(cells.size, nc + w)); ent_c.append(cells * 3 + e); ent_v.append(wwc[w][:, e])
        ent_r.append(np.array([nc + w])); ent_c.append(np.array([nc + w])); ent_v.append(np.array([Dw[w]]))
    R = np.concatenate(ent_r).astype(np.int64)
    Cc = np.concatenate(ent_c).astype(np.int64)
    V = np.concatenate(ent_v)
    ntot = nc + nw
    key = R * ntot + Cc
    order = np.argsort(key, kind="stable")
    uniq, start = np.unique(key[order], return_index=True)
    Vs = np.add.reduceat(V[order], start)
    ur = (uniq // ntot).astype(np.int32)
    uc = (uniq % ntot).astype(np.int32)
    rp = np.zeros(ntot + 1, dtype=np.int64)
    np.add.at(rp, ur + 1, 1)
    rp = np.cumsum(rp).astype(np.int32)
    J = ScalarCSR(rp, uc, Vs)
    xfull = np.concatenate([xt, 50.0 * rng.standard_normal(nw)])
    rows = np.repeat(np.arange(ntot), np.diff(rp))
    bf = np.zeros(ntot)
    np.add.at(bf, rows, Vs * xfull[uc])
    return J, bf


# ---------------------------------------------------------------- named workloads
def run_step(day: float) -> float:
    """The simulator's time step at simulated time `day` on a run reported monthly (tools/gen_bigcase.py: TSTEP
    30.4375): the engine starts at 1 day and doubles the step (Tuning initialDt 1, growth 2), up to the report step."""
    dt, t = 1.0, 0.0
    while t + dt < day:
        t += dt
        dt = min(2.0 * dt, 30.4375)
    return dt


def spe10_like(day: int = 1, seed: int = 0, nx=60, ny=220, nz=85) -> NewtonSystem:
    """60x220x85 SPE10-model-2-sized grid: sigma ln k = 2.5, channels (x100, 4 cells wide) in layers 36-85,
    phi = 0.05 + 0.02 ln k, central injector + 4 corner producers in all layers. ``day`` is the simulated time of the
    Jacobian: the run's own step there (run_step: 1 day on day 1, 30.4 days by day 100) and a water front that has
    grown with the injected volume (radius proportional to the square root of time, half the reservoir scale at
    day 100). Fluxes are upwinded by the flow potential (pressure less the hydrostatic head) of a smooth pressure
    field (0.5 psi cell-to-cell perturbation), as in a simulator's state near equilibrium, so that the vertical
    connections of the thin (2 ft) layers carry only the well-driven flow."""
    return make_system(nx, ny, nz, sigma=2.5, corr=(5, 5, 1), seed=seed, dx=20.0, dy=10.0, dz=2.0,
                       channels=(35, 84, 4, 100.0), wells="corners+center", dt=run_step(day),
                       front_radius=0.5 * math.sqrt(day / 100.0), gravity_head=True, p_noise=0.5)


def ensemble_member(r: int, nx=40, ny=40, nz=10, sigma=1.5, seed0: int = 0, dt: float = 10.0):
    """Realisation r of the ensemble: permeability seed seed0 + r and a seeded inactive fraction U[0.1, 0.5]."""
    frac = float(np.random.default_rng(10_000 + seed0 + r).uniform(0.1, 0.5))
    return make_system(nx, ny, nz, sigma=sigma, seed=seed0 + r, actnum_fraction=frac, wells="corners+center", dt=dt)


def ensemble(n_real: int = 64, nx=40, ny=40, nz=10, sigma=1.5, seed0: int = 0, dt: float = 10.0):
    """Realisations with their own permeability seed and a seeded inactive fraction U[0.1, 0.5]."""
    return [ensemble_member(r, nx, ny, nz, sigma, seed0, dt) for r in range(n_real)]


def black_oil_tables() -> dict:
    """Synthetic black-oil fluid and saturation tables in the layout of the device assembler (ressim_gb300.assembly):
    live oil from Standing's bubble-point correlation and Beggs-Robinson viscosities (API 35, gas gravity 0.8,
    180 F), undersaturated ratio tables, dry gas with a constant z-factor, Corey SWOF / SGOF (Swc = Sor = 0.2,
    exponents 2), field units. A stand-in of the engine's correlation-generated tables for timing the assembly."""
    api, gg, temp = 35.0, 0.8, 180.0
    go = 141.5 / (131.5 + api)
    pb = np.linspace(14.7, 4500.0, 12)
    rs_scf = gg * ((pb / 18.2 + 1.4) * 10 ** (0.0125 * api - 0.00091 * temp)) ** 1.2048
    bo = 0.9759 + 0.000120 * (rs_scf * math.sqrt(gg / go) + 1.25 * temp) ** 1.2
    mu_od = 10 ** (10 ** (3.0324 - 0.02023 * api) * temp ** -1.163) - 1.0
    mu_o = 10.715 * (rs_scf + 100.0) ** -0.515 * mu_od ** (5.44 * (rs_scf + 150.0) ** -0.338)
    rs = rs_scf / 1000.0                                  # Mscf/stb
    dpu = np.array([0.0, 500.0, 1000.0, 2000.0, 5000.0])
    ub_y = 1.0 + 1.0e-5 * dpu
    ubmu_y = (1.0 + 1.0e-5 * dpu) / (1.0 + 4.0e-5 * dpu)
    pg = np.linspace(0.0, 9000.0, 13)
    bg = pg / (5.04 * 0.9 * (temp + 460.0))               # 1/Bg, Mscf/rb
    mug = 0.0125 + 1.0e-6 * pg
    sw = np.linspace(0.2, 1.0, 17)
    swn = np.clip((sw - 0.2) / 0.6, 0.0, 1.0)
    krw = 0.6 * swn ** 2
    krow = np.clip((0.8 - sw) / 0.6, 0.0, 1.0) ** 2
    sg = np.linspace(0.0, 0.8, 17)
    krg = 0.8 * (sg / 0.8) ** 2
    krog = ((0.8 - sg) / 0.8) ** 2
    z = {}

    def tab(name, x, y, clamp):
        z[name + "_x"], z[name + "_y"], z[name + "_clamp"] = np.asarray(x, float), np.asarray(y, float), np.array([clamp], np.int32)

    tab("rsOfP", pb, rs, 0)
    tab("pbOfRs", rs, pb, 0)
    tab("deadB", [], [], 0)
    tab("deadBMu", [], [], 0)
    tab("gasB", pg, bg, 0)
    tab("gasBMu", pg, bg / mug, 0)
    tab("krw", sw, krw, 1)
    tab("krow", sw, krow, 1)
    tab("pcow", sw, np.zeros_like(sw), 1)
    tab("krg", sg, krg, 1)
    tab("krog", sg, krog, 1)
    tab("pcog", sg, np.zeros_like(sg), 1)
    z["liveRs"], z["livePb"], z["bSat"], z["bmuSat"] = rs, pb, 1.0 / bo, 1.0 / (bo * mu_o)
    n = pb.size
    for name, y in (("uB", ub_y), ("uBMu", ubmu_y)):
        z[name + "_x"] = np.tile(dpu, n)
        z[name + "_y"] = np.tile(y, n)
        z[name + "_off"] = (np.arange(n + 1) * dpu.size).astype(np.int32)
        z[name + "_clamp"] = np.zeros(n, np.int32)
    z["phases"] = np.array([1, 1, 1, 1, 0], np.uint8)
    z["vars"] = np.array([1, 2, 0, 1, 2], np.int32)
    z["pvtw"] = np.array([4014.7, 1.029, 3.13e-6, 0.31, 0.0])
    z["rock"] = np.array([14.7, 3.0e-6])
    z["rhoSC"] = np.array([53.0, 64.79, 0.0573])
    z["gasFactor"] = np.array([1000.0 / 5.614583])
    z["gravity"] = np.array([1.0 / 144.0])
    z["swco"] = np.array([0.2])
    z["kroModel"] = np.array([0], np.int32)
    z["sat_flags"] = np.array([1, 1, 0], np.uint8)
    z["fluid_flags"] = np.array([1, 0], np.uint8)
    return z


def assembly_grid(nx, ny, nz, *, sigma=1.5, seed=0, actnum_fraction=0.0, dx=100.0, dy=100.0, dz=20.0, kmean=100.0):
    """The active cells, 7-point connections (transmissibility, depth difference) and pore volumes of make_system's
    grid with the same seed (same permeability field and inactive-cell mask), plus a seeded black-oil state: pressure
    with the hydrostatic gradient, water saturation, free gas (state 1, x = Sg) in the top quarter of the layers and
    undersaturated oil (state 0, x = Rs) below."""
    rng = np.random.default_rng(seed)
    shape = (nz, ny, nx)
    zf = correlated_normal(shape, (5, 5, 1), rng)
    lnk = math.log(kmean) + sigma * zf
    k = np.exp(lnk)
    phi = np.clip(0.05 + 0.02 * lnk, 0.01, 0.45)
    active = np.ones(shape, dtype=bool)
    if actnum_fraction > 0:
        f = correlated_normal(shape, (6, 6, 2), rng)
        active = f > np.quantile(f, actnum_fraction)
    act = active.reshape(-1)
    idx = np.full(act.size, -1, dtype=np.int64)
    na = int(act.sum())
    idx[act] = np.arange(na)
    kf = k.reshape(-1)[act]
    kk_, jj_, ii_ = np.unravel_index(np.nonzero(act)[0], shape)
    depth = 8325.0 + (kk_ + 0.5) * dz
    ca, cb, ct, cd = [], [], [], []
    for (di, dj, dk, area, dist) in ((1, 0, 0, dy * dz, dx), (0, 1, 0, dx * dz, dy), (0, 0, 1, dx * dy, dz)):
        m = np.ones(shape, dtype=bool)
        if di:
            m[:, :, -1] = False
        if dj:
            m[:, -1, :] = False
        if dk:
            m[-1, :, :] = False
        src = np.nonzero(m.reshape(-1))[0]
        a, b_ = idx[src], idx[src + di + dj * nx + dk * nx * ny]
        ok = (a >= 0) & (b_ >= 0)
        a, b_ = a[ok], b_[ok]
        kz = 0.1 if dk else 1.0
        ca.append(a); cb.append(b_)
        ct.append(0.001127 * 2.0 / (1.0 / (kz * kf[a]) + 1.0 / (kz * kf[b_])) * area / dist)
        cd.append(depth[b_] - depth[a])
    pv = phi.reshape(-1)[act] * dx * dy * dz / 5.614583
    p = 4000.0 + 0.45 * (depth - 8325.0) + 200.0 * np.sin(0.1 * ii_) * np.cos(0.08 * jj_) + 5.0 * rng.standard_normal(na)
    sw = np.clip(0.2 + 0.4 * rng.random(na), 0.2, 0.79)
    state = np.where(kk_ < max(1, nz // 4), 1, 0).astype(np.uint8)
    x = np.where(state == 1, 0.02 + 0.1 * rng.random(na), 0.5 + 0.3 * rng.random(na))
    acc_old = np.stack([pv * 0.97 * sw, pv * 0.8 * (1 - sw), pv * (0.8 * (1 - sw) * 0.6 + 0.05)], axis=1).reshape(-1)
    return dict(na=na, ca=np.concatenate(ca), cb=np.concatenate(cb), trans=np.concatenate(ct), dDepth=np.concatenate(cd),
                pv=pv, p=p, sw=sw, x=x, state=state, acc_old=acc_old)


def assembly_model(grids) -> dict:
    """The device assembler's model (ressim_gb300.assembly) of one or more grids taken together as one disconnected
    grid, without wells, and the concatenated state: the engine's scalar Jacobian pattern (cell row a*3+e holds the
    blocks of the cell and its neighbours in column order) and adjacency (per cell, its connections in connection
    order)."""
    ca, cb, tr, dd, pv, st = [], [], [], [], [], {k: [] for k in ("p", "sw", "x", "state", "acc_old")}
    off = 0
    for g in grids:
        ca.append(g["ca"] + off); cb.append(g["cb"] + off)
        tr.append(g["trans"]); dd.append(g["dDepth"]); pv.append(g["pv"])
        for k in st:
            st[k].append(g[k])
        off += g["na"]
    na = off
    ca, cb = np.concatenate(ca).astype(np.int64), np.concatenate(cb).astype(np.int64)
    nconn = ca.size
    # adjacency: every connection from both sides, ordered by cell then connection index
    own = np.concatenate([ca, cb])
    nbr = np.concatenate([cb, ca])
    cid = np.concatenate([np.arange(nconn), np.arange(nconn)])
    o = np.lexsort((cid, own))
    adjStart = np.zeros(na + 1, np.int64)
    np.add.at(adjStart, own + 1, 1)
    adjStart = np.cumsum(adjStart)
    # pattern: per cell its sorted blocks (self and neighbours), three rows with the same columns
    bown = np.concatenate([own, np.arange(na)])
    bnb = np.concatenate([nbr, np.arange(na)])
    ob = np.lexsort((bnb, bown))
    bnb = bnb[ob]
    cnt = np.bincount(bown, minlength=na)
    bstart = np.concatenate([[0], np.cumsum(cnt)])
    cellcols = (3 * bnb[:, None] + np.arange(3)).reshape(-1)
    rowlen = np.repeat(3 * cnt, 3)
    rowPtr = np.concatenate([[0], np.cumsum(rowlen)])
    a_of_row = np.repeat(np.arange(na), 3)
    base = np.repeat(3 * bstart[a_of_row] - rowPtr[:-1], rowlen)
    J_col = cellcols[np.arange(rowPtr[-1]) + base]
    z = black_oil_tables()
    z.update(na=np.array([na]), nv=np.array([3]), nw=np.array([0]), adjStart=adjStart.astype(np.int32),
             adjNbr=nbr[o].astype(np.int32), adjConn=cid[o].astype(np.int32), conn_a=ca.astype(np.int32),
             conn_b=cb.astype(np.int32), conn_trans=np.concatenate(tr), conn_dDepth=np.concatenate(dd),
             poreVolRef=np.concatenate(pv), J_rowPtr=rowPtr.astype(np.int32), J_col=J_col.astype(np.int32))
    state = {k: np.concatenate(v) for k, v in st.items()}
    return z, state


def assembly_ensemble(n_real: int = 64, nx=40, ny=40, nz=10, sigma=1.5, seed0: int = 0):
    """The ensemble's grids (same permeability seeds and inactive-cell masks as ensemble()) as one assembly model."""
    grids = []
    for r in range(n_real):
        frac = float(np.random.default_rng(10_000 + seed0 + r).uniform(0.1, 0.5))
        grids.append(assembly_grid(nx, ny, nz, sigma=sigma, seed=seed0 + r, actnum_fraction=frac))
    return assembly_model(grids)


def serving_request(rng: np.random.Generator, cells_lo=1e3, cells_hi=1e6, max_cells=None) -> NewtonSystem:
    """One serving request: log-uniform cell count, random box with nz in [1, 50], sigma ln k in [0.5, 3],
    time step in [0.1, 30] days, 1-8 wells."""
    hi = cells_hi if max_cells is None else min(cells_hi, max_cells)
    ncell = int(round(math.exp(rng.uniform(math.log(cells_lo), math.log(hi)))))
    nz = int(rng.integers(1, 51))
    nz = max(1, min(nz, ncell))
    area = max(1, ncell // nz)
    asp = math.exp(rng.uniform(-1.0, 1.0))
    nx = max(1, int(round(math.sqrt(area * asp))))
    ny = max(1, area // nx)
    return make_system(nx, ny, nz, sigma=float(rng.uniform(0.5, 3.0)), seed=int(rng.integers(0, 2**31 - 1)),
                       dt=float(rng.uniform(0.1, 30.0)), wells="random", n_wells=int(rng.integers(1, 9)))


def make_block_system(nx, ny, nz, nb, *, sigma=1.0, seed=0, dt=5.0, well_columns=2) -> NewtonSystem:
    """A Newton system with nb unknowns per cell (pressure first, then nb - 1 transported quantities: component
    moles of a compositional model, or saturations and temperature of a thermal one), for the block-size-generic
    path. Same structure as ``make_system``: 7-point TPFA connections with harmonic-mean transmissibilities of a
    log-normal permeability, upstream-weighted mobilities of every equation with their derivatives in the transported
    unknowns, accumulation blocks scaled by PV / dt (the true-IMPES ``acc``), and ``well_columns`` columns of cells
    coupled to each other (the fill a well's Schur complement adds), so that some rows carry more than the stencil's
    seven blocks. b = S x_true with a manufactured x_true."""
    rng = np.random.default_rng(seed)
    shape = (nz, ny, nx)
    k = np.exp(math.log(100.0) + sigma * correlated_normal(shape, (5, 5, 1), rng)).reshape(-1)
    n = nx * ny * nz
    kk_, jj_, ii_ = np.unravel_index(np.arange(n), shape)
    p = 3000.0 + 0.45 * 20.0 * (kk_ + 0.5) - 300.0 * np.exp(-np.hypot(ii_ - nx / 2.0, jj_ - ny / 2.0) / max(nx, ny))
    mob = rng.uniform(0.2, 1.0, size=(n, nb))                # mobility of every equation's quantity
    dmob = 0.05 * rng.standard_normal(size=(n, nb, nb - 1))  # its derivative in the transported unknowns
    pv = 0.2 * 100.0 * 100.0 * 20.0 / 5.615
    acc = np.zeros((n, nb, nb))
    acc[:, :, 0] = 0.05 * rng.uniform(0.5, 1.5, size=(n, nb))     # compressibility terms
    acc[:, :, 1:] = 0.1 * rng.standard_normal(size=(n, nb, nb - 1))
    for e in range(1, nb):
        acc[:, e, e] += 1.0
    acc[:, 0, 1:] += 0.5 / (nb - 1)                            # the pressure equation sums the quantities
    scale = dt / pv
    conns = []
    for (di, dj, dk, area, dist, kz) in ((1, 0, 0, 2000.0, 100.0, 1.0), (0, 1, 0, 2000.0, 100.0, 1.0), (0, 0, 1, 1e4, 20.0, 0.1)):
        m = np.ones(shape, dtype=bool)
        if di:
            m[:, :, -1] = False
        if dj:
            m[:, -1, :] = False
        if dk:
            m[-1, :, :] = False
        a = np.nonzero(m.reshape(-1))[0]
        b_ = a + di + dj * nx + dk * nx * ny
        kh = 2.0 / (1.0 / (kz * k[a]) + 1.0 / (kz * k[b_]))
        conns.append((a, b_, 0.001127 * kh * area / dist))
    ca = np.concatenate([c[0] for c in conns])
    cb = np.concatenate([c[1] for c in conns])
    T = np.concatenate([c[2] for c in conns])
    dp = p[cb] - p[ca]
    up = np.where(dp < 0, ca, cb)
    ua = (up == ca)[:, None, None]
    nc = ca.size
    blk_ab = np.zeros((nc, nb, nb))
    blk_ab[:, :, 0] = -(T[:, None] * mob[up])
    dS = -(T * dp)[:, None, None] * dmob[up]
    blk_ab[:, :, 1:] += np.where(ua, 0.0, dS)
    blk_aa = np.zeros((nc, nb, nb))
    blk_aa[:, :, 0] = T[:, None] * mob[up]
    blk_aa[:, :, 1:] += np.where(ua, dS, 0.0)
    diag = acc.copy()
    np.add.at(diag, ca, scale * blk_aa)
    np.add.at(diag, cb, scale * blk_aa)
    rows, cols, vals = [np.arange(n), ca, cb], [np.arange(n), cb, ca], [diag, scale * blk_ab, scale * blk_ab]
    for w in range(well_columns):
        i0, j0 = int(rng.integers(0, nx)), int(rng.integers(0, ny))
        cells = (np.arange(nz) * ny + j0) * nx + i0
        m = cells.size
        f = 0.05 * rng.standard_normal(size=(m, m, nb, nb)) * scale
        rows.append(np.repeat(cells, m)); cols.append(np.tile(cells, m)); vals.append(f.reshape(m * m, nb, nb))
    R = np.concatenate(rows).astype(np.int64)
    Cc = np.concatenate(cols).astype(np.int64)
    V = np.concatenate(vals, axis=0)
    key = R * n + Cc
    order = np.argsort(key, kind="stable")
    uniq, start = np.unique(key[order], return_index=True)
    Vs = np.add.reduceat(V[order], start, axis=0)
    ur = (uniq // n).astype(np.int32)
    rowPtr = np.zeros(n + 1, dtype=np.int64)
    np.add.at(rowPtr, ur + 1, 1)
    A = BSR(n, nb, np.cumsum(rowPtr).astype(np.int32), (uniq % n).astype(np.int32), Vs.reshape(-1))
    xt = rng.standard_normal(n * nb)
    xt[0::nb] *= 20.0
    b = bsr_matvec_host(A, xt)
    return NewtonSystem(A, b, acc=acc.reshape(-1), na=n, nv=nb, nw=0, x_true=xt,
                        meta=dict(nx=nx, ny=ny, nz=nz, nb=nb, sigma=sigma, seed=seed, dt=dt))
