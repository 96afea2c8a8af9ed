"""Learned warm start of steady 2-D D2Q9 cases (no counterpart in the
reference).

Cases: lid-driven cavities (MovingWall lid at y = hi, NoSlip elsewhere) and
channels (Inflow at x = lo, PressureOutlet at x = hi, NoSlip at y = lo, hi),
n x n cells, Re uniform in [100, 2000] (Re = U n / nu), lid / inflow velocity
U uniform in [0.02, 0.1], tau = 0.5 + 3 U n / Re, and 0-3 seeded solid boxes
covering 5-20 % of the domain in total.

The plain solver (a batch of all cases, one kernel per step, FP64-accurate
fixed-point storage) produces the steady fields: a case is steady when the
relative change of its stored-population velocity over 100 steps drops
below `tol` (1e-8).  The surrogate
(surrogate.UNet) learns (rho, u) from the geometry and parameters; a warm
start initialises f = feq + f_neq(grad u) from its prediction
(mph_init_fields_neq), and the same solver iterates to the same residual.
"""
from __future__ import annotations

import math
import time

import numpy as np

from . import Batch, MphError, lattice_tables, make_desc, set_device

RE = (100.0, 2000.0)
U = (0.02, 0.1)


def draw_cases(n_cases, seed, sizes=(128,), kinds=("cavity", "channel")):
    rng = np.random.default_rng(seed)
    cases = []
    while len(cases) < n_cases:
        n = int(sizes[len(cases) % len(sizes)])
        kind = kinds[int(rng.integers(len(kinds)))]
        re = float(rng.uniform(*RE))
        u = float(rng.uniform(*U))
        tau = 0.5 + 3.0 * u * n / re
        nbox = int(rng.integers(0, 4))
        frac = float(rng.uniform(0.05, 0.20)) if nbox else 0.0
        boxes = []
        if nbox:
            area = frac * n * n / nbox
            for _ in range(nbox):
                aspect = math.exp(rng.uniform(math.log(0.4), math.log(2.5)))
                w = int(max(2, min(n // 2, round(math.sqrt(area * aspect)))))
                h = int(max(2, min(n // 2, round(area / w))))
                # keep a fluid margin of 3 cells to the faces
                x0 = int(rng.integers(3, max(4, n - w - 3)))
                y0 = int(rng.integers(3, max(4, n - h - 3)))
                boxes.append((x0, y0, w, h))
        cases.append({"kind": kind, "n": n, "Re": re, "U": u, "tau": tau, "boxes": boxes})
    return cases


def case_mask(c):
    n = c["n"]
    m = np.zeros((n, n), np.uint8)  # [y][x]
    for x0, y0, w, h in c["boxes"]:
        m[y0:y0 + h, x0:x0 + w] = 1
    return m


def case_desc(c, precision="f32"):
    n, u = c["n"], c["U"]
    U6 = [[0.0] * 3 for _ in range(6)]
    if c["kind"] == "cavity":
        faces = ["NoSlip", "NoSlip", "NoSlip", "MovingWall", "Periodic", "Periodic"]
        U6[3] = [u, 0.0, 0.0]
    else:
        faces = ["Inflow", "PressureOutlet", "NoSlip", "NoSlip", "Periodic", "Periodic"]
        U6[0] = [u, 0.0, 0.0]
    return make_desc("D2Q9", (n, n), 1.0 / c["tau"], faces=faces, face_U=U6, precision=precision)


def features(c):
    """Network input [n][n][8]: solid, driving face, no-slip face, outlet
    face, normalised log Re, U / 0.1, x, y."""
    n = c["n"]
    f = np.zeros((n, n, 8), np.float32)
    f[..., 0] = case_mask(c)
    if c["kind"] == "cavity":
        f[-1, :, 1] = 1.0
        f[0, :, 2] = f[:, 0, 2] = f[:, -1, 2] = 1.0
    else:
        f[:, 0, 1] = 1.0
        f[0, :, 2] = f[-1, :, 2] = 1.0
        f[:, -1, 3] = 1.0
    f[..., 4] = (math.log(c["Re"]) - math.log(RE[0])) / (math.log(RE[1]) - math.log(RE[0]))
    f[..., 5] = c["U"] / U[1]
    t = (np.arange(n, dtype=np.float32) + 0.5) / n
    f[..., 6] = t[None, :]
    f[..., 7] = t[:, None]
    return f


def rho_scale(c):
    """Scale of rho - 1: inertial (3 U^2) plus viscous (36 nu U / n)."""
    nu = (c["tau"] - 0.5) / 3.0
    return 3.0 * c["U"] ** 2 + 36.0 * nu * c["U"] / c["n"]


def targets(c, rho, u):
    n = c["n"]
    t = np.empty((n, n, 3), np.float32)
    t[..., 0] = ((rho.reshape(n, n) - 1.0) / rho_scale(c))
    t[..., 1] = u[: n * n].reshape(n, n) / c["U"]
    t[..., 2] = u[n * n:].reshape(n, n) / c["U"]
    return t


def fields_from_prediction(c, pred):
    """(rho, u) in the solver's layout from a [n][n][3] prediction."""
    n = c["n"]
    solid = case_mask(c).reshape(-1).astype(bool)
    rho = 1.0 + rho_scale(c) * pred[..., 0].astype(np.float64).reshape(-1)
    u = np.concatenate([pred[..., 1].reshape(-1), pred[..., 2].reshape(-1)]).astype(np.float64) * c["U"]
    rho[solid] = 1.0
    u[: n * n][solid] = 0.0
    u[n * n:][solid] = 0.0
    return rho, u


def _batch(cases, precision):
    b = Batch([case_desc(c, precision) for c in cases])
    for i, c in enumerate(cases):
        b.set_obstacles(i, case_mask(c))
    return b


def _feq_d2q9(rho, u, n):
    """Equilibrium populations [9][n*n] of (rho, u) (D2Q9, u = [ux..., uy...])."""
    c, w, _ = lattice_tables("D2Q9")
    ux, uy = u[: n * n], u[n * n:]
    usq = ux * ux + uy * uy
    cu = c[:, 0:1] * ux[None, :] + c[:, 1:2] * uy[None, :]
    return w[:, None] * rho[None, :] * (1.0 + 3.0 * cu + 4.5 * cu * cu - 1.5 * usq[None, :])


def _moments_d2q9(f, n):
    """(rho, u) of populations f [9][n*n] (D2Q9, u = [ux..., uy...])."""
    c, _, _ = lattice_tables("D2Q9")
    f = f.reshape(9, n * n)
    rho = f.sum(axis=0)
    u = np.concatenate([(c[:, 0:1] * f).sum(axis=0), (c[:, 1:2] * f).sum(axis=0)])
    return rho, u / np.tile(rho, 2)


def consistent_start(b, cases, idx, targets, steps=20, rounds=3):
    """Make the non-equilibrium part of warm-started batch domains consistent
    with the solver (an approach in the spirit of Mei et al., Computers &
    Fluids 35 (2006), consistent initial conditions for lattice Boltzmann):
    `rounds` times, advance `steps` steps, then put back the prescribed (rho,
    u) of each domain while keeping the non-equilibrium part f - feq(rho_f,
    u_f) the solver has built.  Solid cells keep the rest state.  Returns the
    steps spent."""
    _, w, _ = lattice_tables("D2Q9")
    for _ in range(rounds):
        try:
            b.advance(steps)
        except MphError as ex:  # a diverging fixed-point domain is flagged; the others stepped
            if ex.code != 6:
                raise
        for j, i in enumerate(idx):
            c = cases[i]
            n = c["n"]
            f = b.f(j).reshape(9, n * n)
            rho_f, u_f = _moments_d2q9(f, n)
            rho_t, u_t = targets[i]
            g = _feq_d2q9(rho_t, u_t, n) + (f - _feq_d2q9(rho_f, u_f, n))
            solid = case_mask(c).reshape(-1).astype(bool)
            if solid.any():
                g[:, solid] = w[:, None]
            b.set_f(j, g.reshape(-1))
    return steps * rounds


def solve(cases, init=None, max_steps=400_000, tol=1e-8, check_every=1000, k=100, log=None, precision="f64x",
          compact=0.6, consistent=None):
    """Advance all cases together from rest (init None) or from
    init[i] = (rho, u) (warm start), until each reaches the residual tol over
    k steps.  The default storage is the FP64-accurate fixed point (FP32
    storage stalls near a residual of 1e-6).  A fixed-point case whose
    populations leave the representable range (an unstable high-Re case)
    counts as diverged; the other cases step on.  Cases that converge or
    diverge leave the batch: once at most `compact` of a batch's domains still run,
    the running ones move into a new batch (populations carried over at FP64
    resolution through mph_batch_set_f), so late cases do not pay for early
    ones.  consistent = (steps, rounds): after a warm start, first make the
    non-equilibrium part consistent (consistent_start); its steps count
    towards every case's steps.  Returns (steps per case: -1 not reached, -2
    diverged; (rho, u) per case when it stopped; seconds; last residual per
    case)."""
    set_device(0)
    n_all = len(cases)
    steps = np.full(n_all, -1, np.int64)
    last = np.full(n_all, np.inf)
    out = [None] * n_all
    t0 = time.perf_counter()
    idx = list(range(n_all))  # global index of each batch domain
    b = _batch(cases, precision)
    for j, c in enumerate(cases):
        if init is None:
            b.initialize(j)
        else:
            b.initialize_neq(j, *init[j])
    def advance(nsteps):
        try:
            b.advance(nsteps)
        except MphError as ex:
            if ex.code != 6:  # MPH_ERR_NONFINITE: flagged domains report NaN residuals
                raise

    done = 0
    if init is not None and consistent:
        done = consistent_start(b, cases, idx, init, *consistent)
    while done < max_steps and np.any(steps[idx] == -1):
        advance(check_every - k)
        b.residual()
        advance(k)
        r, _ = b.residual()
        done += check_every
        for j, i in enumerate(idx):
            if steps[i] != -1:
                continue
            last[i] = r[j]
            if np.isnan(r[j]):
                steps[i] = -2  # diverged
                out[i] = b.moments(j)
            elif r[j] < tol:
                steps[i] = done
                out[i] = b.moments(j)
        running = [j for j, i in enumerate(idx) if steps[i] == -1]
        if log:
            log(done, int(np.sum(steps > 0)), float(np.nanmedian(last)), len(idx))
        if running and len(running) <= compact * len(idx) and done < max_steps:
            fs = [b.f(j) for j in running]
            b.close()
            idx = [idx[j] for j in running]
            b = _batch([cases[i] for i in idx], precision)
            for j, f in enumerate(fs):
                b.set_f(j, f)
    for j, i in enumerate(idx):
        if out[i] is None:
            out[i] = b.moments(j)
    secs = time.perf_counter() - t0
    b.close()
    return steps, out, secs, last


def smooth_field(n, rng, modes=3):
    """A smooth random field on n x n cells: a sum of products of sines with
    wave numbers 1..modes along each axis and random amplitudes and phases."""
    t = (np.arange(n) + 0.5) / n
    f = np.zeros((n, n))
    for kx in range(1, modes + 1):
        for ky in range(1, modes + 1):
            a = rng.standard_normal() / (kx * ky)
            px, py = rng.uniform(0, 2 * np.pi, 2)
            f += a * np.sin(np.pi * ky * t + py)[:, None] * np.sin(np.pi * kx * t + px)[None, :]
    return f


def perturbed_fields(c, rho, u, e, rng):
    """(rho, u) of a converged case with smooth noise of relative L2 amplitude
    e in u over the fluid cells (and e times the rho - 1 scale in rho);
    solid cells keep the rest state."""
    n = c["n"]
    fluid = case_mask(c).reshape(-1) == 0
    phi = np.concatenate([smooth_field(n, rng).reshape(-1), smooth_field(n, rng).reshape(-1)])
    phi[np.tile(~fluid, 2)] = 0.0
    uf = np.tile(fluid, 2)
    du = e * np.linalg.norm(u[uf]) / max(np.linalg.norm(phi[uf]), 1e-300) * phi
    pr = smooth_field(n, rng).reshape(-1)
    pr[~fluid] = 0.0
    drho = e * rho_scale(c) * pr / max(np.sqrt(np.mean(pr[fluid] ** 2)), 1e-300)
    return rho + drho, u + du


def perturbation_curve(cases, fields, amps, seed=0, consistent=None, **solve_kw):
    """Steps to the residual tol from the converged fields of `cases` with
    smooth noise of each relative amplitude in `amps` (0 = the converged
    field itself through feq + f_neq), and from rest, all in one batch.
    Returns {amp: steps per case} with the key 'rest' for the start from rest."""
    rng = np.random.default_rng(seed)
    run_cases, inits, keys = [], [], []
    for c, (rho, u) in zip(cases, fields):
        for e in amps:
            run_cases.append(c)
            inits.append(perturbed_fields(c, rho, u, e, rng))
            keys.append(e)
    steps, _, secs, _ = solve(run_cases, inits, consistent=consistent, **solve_kw)
    plain, _, secs_rest, _ = solve(cases, None, **solve_kw)
    table = {e: [int(s) for s, k in zip(steps, keys) if k == e] for e in amps}
    table["rest"] = [int(s) for s in plain]
    return table, secs + secs_rest


def dataset(cases, fields, limit=20.0):
    """Network arrays of the cases with finite, bounded targets (|t| <= limit;
    larger values mean a field far from a steady state at this scale):
    X [S][n][n][8], Y [S][n][n][3], fluid mask M [S][n][n]."""
    X, Y, M = [], [], []
    for c, (rho, u) in zip(cases, fields):
        t = targets(c, rho, u)
        if not np.all(np.isfinite(t)) or np.max(np.abs(t)) > limit:
            continue
        X.append(features(c))
        Y.append(t)
        M.append(1.0 - case_mask(c).astype(np.float32))
    return np.stack(X), np.stack(Y), np.stack(M)


def mirror_channels(X, Y, M):
    """Channels are symmetric under y -> n - 1 - y (uniform inflow, walls at
    both y faces): append the mirrored copy of every channel sample (obstacles
    mirrored, u_y negated) to the training arrays."""
    ch = X[..., 3].max(axis=(1, 2)) > 0  # the outlet column marks a channel
    if not ch.any():
        return X, Y, M
    Xm = X[ch][:, ::-1].copy()
    Xm[..., 7] = X[ch][..., 7]  # the y coordinate channel keeps its orientation
    Ym = Y[ch][:, ::-1].copy()
    Ym[..., 2] = -Ym[..., 2]
    Mm = M[ch][:, ::-1].copy()
    return np.concatenate([X, Xm]), np.concatenate([Y, Ym]), np.concatenate([M, Mm])


def train(X, Y, M, epochs=30, batch=8, lr=1e-3, seed=0, log=None, net=None, clip=1.0):
    """Adam with a cosine learning-rate schedule and global gradient-norm
    clipping over shuffled mini-batches; returns (net, per-epoch mean loss)."""
    from .surrogate import Trainer, UNet
    S, n = X.shape[0], X.shape[1]
    net = net or UNet(seed=seed)
    tr = Trainer(net, batch, n, n)
    rng = np.random.default_rng(seed)
    total = epochs * (S // batch)
    it, hist = 0, []
    for ep in range(epochs):
        order = rng.permutation(S)
        losses = []
        for j in range(S // batch):
            idx = order[j * batch:(j + 1) * batch]
            lr_t = 0.5 * lr * (1.0 + math.cos(math.pi * it / total))
            losses.append(tr.train_step(X[idx], Y[idx], M[idx], lr_t, clip=clip))
            it += 1
        hist.append(float(np.mean(losses)))
        if log:
            log(ep, hist[-1])
    return net, hist


def predict(net, cases, batch=8):
    """(rho, u) predictions in the solver's layout, and the seconds taken."""
    from .surrogate import Trainer
    n = cases[0]["n"]
    tr = Trainer(net, batch, n, n)
    out = []
    t0 = time.perf_counter()
    for j in range(0, len(cases), batch):
        cs = cases[j:j + batch]
        pred = tr.predict(np.stack([features(c) for c in cs]))
        out.extend(fields_from_prediction(c, p) for c, p in zip(cs, pred))
    return out, time.perf_counter() - t0


def field_error(c, pred, ref):
    """Relative L2 error of the predicted velocity over the fluid cells."""
    fluid = np.tile(case_mask(c).reshape(-1) == 0, 2)
    du = (pred[1] - ref[1])[fluid]
    return float(np.linalg.norm(du) / max(np.linalg.norm(ref[1][fluid]), 1e-30))
