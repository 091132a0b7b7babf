"""The learned PV-on-edge closure: training data, training, and ensembles
with a per-member invariant-drift fallback.

Training data: FP64 runs of the fine mesh (seeded jet + mountains), sampled
at intervals and coarse-grained on the device (``Coarsener``); the coarse FP32
model is set to each coarse-grained state and exports its closure features
and its own pv on edges; the target is the coarse-grained fine pv on edges
minus the coarse model's (the PV-on-edge residual).  Training is Adam on the
device (``ClosureMLP``).  Inference runs inside the FP32 step of an ensemble
(``TMCoreGPU.set_closure``); ``FallbackMonitor`` switches the closure off for
a member whose total energy or mass drifts beyond a bound and restores that
member's last checkpoint.

Run ``python -m tmcore_gb300.closure --help`` for the end-to-end pipeline.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np

from . import abi, cases
from .gpu import ClosureMLP, Coarsener, TMCoreGPU
from .mesh import icos_mesh

DAY = 86400.0


def level_dt(level: int) -> float:
    """dt = 1200 / 2^(level - 4) s."""
    return 1200.0 / 2 ** (level - 4)


def _edge_pv(mesh, pv_vertex):
    v1, v2 = mesh.verticesOnEdge[:, 0] - 1, mesh.verticesOnEdge[:, 1] - 1
    return 0.5 * (pv_vertex[v1] + pv_vertex[v2])


def _jet_bumps_ic(job):
    """Initial state of one seeded run (runs in a spawned worker)."""
    level, seed = job
    return cases.jet_bumps(icos_mesh(level), seed=seed)


def _ics(level, seeds):
    """Seeded initial states, in order, from a spawn pool (safe beside CUDA work)."""
    import multiprocessing as mp
    import os

    jobs = [(level, s) for s in seeds]
    if level <= 6 or len(jobs) < 4:  # a fraction of a second each: no pool
        yield from map(_jet_bumps_ic, jobs)
        return
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1, len(jobs))) as pool:
        yield from pool.imap(_jet_bumps_ic, jobs)


def training_data(fine_level=8, coarse_level=6, runs=4, days=1.0, samples_per_run=8, seed0=0, device=0,
                  log=None, truth="fp64", edge_frac=1.0, skipped=None):
    """(features [N, 24] float32, targets [N] float32) from fine runs.

    truth="fp64": FP64 runs, one at a time.  truth="fp32": all runs as one
    FP32 ensemble (member-innermost when `runs` is a multiple of 16: FP32 edge
    and vertex state, double-float gd), the way many runs fit the budget;
    its difference from FP64 is measured by `evaluate(truth_check=...)`.
    edge_frac < 1 keeps that fraction of each sample's coarse edges (seeded
    random subset) to bound the dataset's size.  A run no longer finite at a
    sample (the dycore has no diffusion) gives no rows there; `skipped`, a
    list, receives its (run, sample) pairs."""
    fine, coarse = icos_mesh(fine_level), icos_mesh(coarse_level)
    dt_f = level_dt(fine_level)
    steps = max(1, int(round(days * DAY / dt_f / samples_per_run)))
    kw = dict(pv_scheme=1, apvm_weight=0.0, adv_order=2, conserve_energy=1, renumber=1, device=device)
    ne_c = coarse.dims["nEdges"]
    keep = max(1, int(round(edge_frac * ne_c)))
    n_rows = runs * samples_per_run * keep
    X = np.empty((n_rows, 24), np.float32)
    Y = np.empty(n_rows, np.float32)
    rng = np.random.default_rng(seed0 + 7)
    cg = Coarsener(fine, coarse, device=device)
    cm = TMCoreGPU(coarse, dt=level_dt(coarse_level), precision=abi.TMC_FP32, **kw)
    row = 0

    if skipped is None:
        skipped = []  # (run, sample) of fine states that are no longer finite

    def add_sample(gdf, uf, pvv, ghs_c, r, s):
        nonlocal row
        if not (np.all(np.isfinite(gdf)) and np.all(np.isfinite(uf)) and np.all(np.isfinite(pvv))):
            skipped.append((r, s))
            return
        gd_c, u_c, pv_true = cg(gd=gdf, u=uf, pv_edge=_edge_pv(fine, pvv))
        cm.set_initial(gd_c, u_c, ghs_c)
        x, pv_c = cm.closure_features()
        y = (pv_true - pv_c).astype(np.float32)
        if not (np.all(np.isfinite(x)) and np.all(np.isfinite(y))):
            skipped.append((r, s))
            return
        idx = np.sort(rng.choice(ne_c, keep, replace=False)) if keep < ne_c else slice(None)
        X[row:row + keep] = x[idx]
        Y[row:row + keep] = y[idx]
        row += keep
        if log and (truth == "fp64" or r % 16 == 0):
            log(f"run {r} sample {s}: |residual| {np.sqrt(np.mean(y ** 2)):.3e}")

    if truth == "fp64":
        for r, (gd, u, ghs) in enumerate(_ics(fine_level, range(seed0, seed0 + runs))):
            fm = TMCoreGPU(fine, dt=dt_f, precision=abi.TMC_FP64, diag_every=0, **kw)
            fm.set_initial(gd, u, ghs)
            ghs_c, _, _ = cg(gd=ghs)
            for s in range(samples_per_run):
                fm.step(steps)
                gdf, _, uf = fm.get_state()
                pvv, _ = fm.get_vertex()
                add_sample(gdf, uf, pvv, ghs_c, r, s)
            fm.close()
    else:
        fm = TMCoreGPU(fine, dt=dt_f, precision=abi.TMC_FP32, diag_every=0, members=runs,
                       member_layout=1 if runs % 16 == 0 else 0, **kw)
        ghs_c = []
        for r, (gd, u, ghs) in enumerate(_ics(fine_level, range(seed0, seed0 + runs))):
            fm.select_member(r)
            fm.set_initial(gd, u, ghs)
            ghs_c.append(cg(gd=ghs)[0])
        for s in range(samples_per_run):
            fm.step(steps)
            for r in range(runs):
                fm.select_member(r)
                gdf, _, uf = fm.get_state()
                pvv, _ = fm.get_vertex()
                add_sample(gdf, uf, pvv, ghs_c[r], r, s)
        fm.close()
    cm.close()
    cg.close()
    if skipped and log:
        runs_lost = sorted({r for r, _ in skipped})
        log(f"{len(skipped)} samples of {len(runs_lost)} runs skipped (state not finite): runs {runs_lost[:20]}")
    return X[:row], Y[:row]


def train(X, Y, steps=2000, batch=65536, lr=1e-3, seed=0, device=0, tensor_cores=True, head=2, dt=None):
    """A ClosureMLP fitted to (X, Y), its gradients on the tensor cores (or
    the CUDA cores); returns (net, losses, scaling).

    head 2 (the default) fits the residual where the correction has APVM's
    sign along the edge (it removes potential enstrophy through q.F_perp
    there) and applies nothing elsewhere; head 1 fits a non-negative per-edge
    APVM weight (the correction is -softplus(y) dt (v dq/dt + u dq/dn), dt the
    coarse model's time step); head 0 fits the residual itself, unconstrained."""
    if head == 1 and not dt:
        raise ValueError("the APVM head needs the coarse model's time step dt")
    rng = np.random.default_rng(seed)
    perm = rng.permutation(len(Y))
    X, Y = X[perm], Y[perm]
    xm = X.mean(0).astype(np.float64)
    xs = X.std(0).astype(np.float64)
    xs[xs == 0] = 1.0
    ys = float(np.std(Y)) or 1.0
    net = ClosureMLP(device=device, seed=seed)
    net.set_train_mode(tensor_cores)
    net.set_scaling(xm, 1.0 / xs, ys)
    net.set_head(head, dt or 0.0)
    net.set_dataset(X, Y)
    b = min(batch, (len(Y) // 128) * 128)
    losses = net.train(steps=steps, batch=b, lr=lr)
    return net, losses, {"x_mean": xm, "x_inv_std": 1.0 / xs, "y_scale": ys, "head": head, "head_dt": dt or 0.0}


def save(path, net, scaling):
    np.savez(path, params=net.params, **scaling)


def load(path, device=0):
    z = np.load(path)
    net = ClosureMLP(device=device)
    net.params = z["params"]
    net.set_scaling(z["x_mean"], z["x_inv_std"], float(z["y_scale"]))
    if "head" in z:
        net.set_head(int(z["head"]), float(z["head_dt"]))
    return net


def _rel_l2(a, b, w):
    return float(np.sqrt(np.sum(w * (a - b) ** 2) / np.sum(w * b * b)))


def _member_states(model, members):
    out = []
    for k in range(members):
        model.select_member(k)
        gd, _, u = model.get_state()
        out.append((gd, u))
    return out


def evaluate(net, fine_level=7, coarse_level=5, members=8, days=5.0, samples=5, seed0=10_000, device=0,
             log=None, truth="fp64", apvm_weight=0.5, truth_check=0):
    """Held-out comparison of the learned coarse run with the plain method.

    `net` is a ClosureMLP (runs "closure", every stage, and "closure_stage1",
    stage 1 held), or a dict {name: ClosureMLP}, each run in stage 1 held.

    For `members` seeds not used in training, the run on the fine mesh,
    coarse-grained onto the coarse mesh, is the truth: FP64 runs one member at
    a time (truth="fp64"), or one FP32 ensemble of all members (truth="fp32",
    member-innermost when members is a multiple of 16; its difference from
    FP64 is far below the coarse runs' errors).  FP32 ensembles start from the
    coarse-grained initial state: the coarse mesh with the closure in every
    stage ("closure"), the same with the closure run in stage 1 and its output
    held for the other stages ("closure_stage1"), the coarse mesh without it
    ("plain"), the coarse mesh with the reference's APVM at a fixed weight
    ("apvm", pv_scheme 1 with `apvm_weight`; omitted when 0), and the plain
    method one level finer ("plain_finer", coarse-grained onto the coarse mesh
    for scoring).  With truth="fp32" and truth_check = k > 0, the first k
    members are also run in FP64 and the relative L2 difference of the two
    coarse-grained truths is reported per sample ("truth_fp32_vs_fp64").  At `samples` evenly spaced times each gets the member-mean
    relative L2 error of h (area weighted) and of u (dvEdge dcEdge weighted);
    each gets its device time per simulated day (CUDA events around its
    steps, all members).
    """
    fine, coarse, mid = icos_mesh(fine_level), icos_mesh(coarse_level), icos_mesh(coarse_level + 1)
    kw = dict(pv_scheme=1, apvm_weight=0.0, adv_order=2, conserve_energy=1, renumber=1, device=device)
    lay = dict(member_layout=1) if members % 16 == 0 else {}
    cg_c, cg_m = Coarsener(fine, coarse, device=device), Coarsener(fine, mid, device=device)
    cg_mc = Coarsener(mid, coarse, device=device)
    dt_f, dt_c, dt_m = level_dt(fine_level), level_dt(coarse_level), level_dt(coarse_level + 1)
    total = days * DAY
    n_f = int(round(total / samples / dt_f))
    n_c, n_m = int(round(total / samples / dt_c)), int(round(total / samples / dt_m))
    ens = dict(members=members, precision=abi.TMC_FP32, diag_every=0, **lay)
    nets = net if isinstance(net, dict) else {"closure": net, "closure_stage1": net}
    runs = {name: TMCoreGPU(coarse, dt=dt_c, **ens, **kw) for name in nets}
    runs["plain"] = TMCoreGPU(coarse, dt=dt_c, **ens, **kw)
    if apvm_weight > 0:  # APVM runs in the member-outermost layout
        runs["apvm"] = TMCoreGPU(coarse, dt=dt_c, **dict(ens, member_layout=0), **dict(kw, apvm_weight=apvm_weight))
    runs["plain_finer"] = TMCoreGPU(mid, dt=dt_m, **ens, **kw)
    ref = [[None] * samples for _ in range(members)]  # per member: truth (gd, u) on the coarse mesh per sample
    fine_ics = []
    for k in range(members):
        gd, u, ghs = cases.jet_bumps(fine, seed=seed0 + k)
        fine_ics.append((gd, u, ghs))
        for name, r in runs.items():
            cg = cg_m if name == "plain_finer" else cg_c
            gd0, u0, _ = cg(gd=gd, u=u)
            ghs0, _, _ = cg(gd=ghs)
            r.select_member(k)
            r.set_initial(gd0, u0, ghs0)
    truth_is_fp64 = truth == "fp64"
    if truth_is_fp64:
        for k, (gd, u, ghs) in enumerate(fine_ics):
            fm = TMCoreGPU(fine, dt=dt_f, precision=abi.TMC_FP64, diag_every=0, **kw)
            fm.set_initial(gd, u, ghs)
            for s in range(samples):
                fm.step(n_f)
                gdf, _, uf = fm.get_state()
                ref[k][s] = cg_c(gd=gdf, u=uf)[:2]
            fm.close()
    else:
        fm = TMCoreGPU(fine, dt=dt_f, **ens, **kw)
        for k, (gd, u, ghs) in enumerate(fine_ics):
            fm.select_member(k)
            fm.set_initial(gd, u, ghs)
        for s in range(samples):
            fm.step(n_f)
            for k in range(members):
                fm.select_member(k)
                gdf, _, uf = fm.get_state()
                ref[k][s] = cg_c(gd=gdf, u=uf)[:2]
        fm.close()
    check = {"h": [[] for _ in range(samples)], "u": [[] for _ in range(samples)]}
    wa0, we0 = coarse.vars["areaCell"], coarse.vars["dvEdge"] * coarse.vars["dcEdge"]
    for k in range(min(truth_check, members) if not truth_is_fp64 else 0):
        gd, u, ghs = fine_ics[k]
        fm = TMCoreGPU(fine, dt=dt_f, precision=abi.TMC_FP64, diag_every=0, **kw)
        fm.set_initial(gd, u, ghs)
        for s in range(samples):
            fm.step(n_f)
            gdf, _, uf = fm.get_state()
            g64, u64 = cg_c(gd=gdf, u=uf)[:2]
            check["h"][s].append(_rel_l2(ref[k][s][0], g64, wa0))
            check["u"][s].append(_rel_l2(ref[k][s][1], u64, we0))
        fm.close()
    fine_ics = None
    for name, n in nets.items():
        runs[name].set_closure(n)
        # "closure" runs the network in every stage; the others in stage 1, held
        runs[name].set_closure_stages(name == "closure")
    wa = coarse.vars["areaCell"]
    we = coarse.vars["dvEdge"] * coarse.vars["dcEdge"]
    err = {name: {"h": [], "u": [], "nonfinite": []} for name in runs}
    ms = {name: 0.0 for name in runs}
    truth_members = []
    for s in range(samples):
        # members whose truth is still finite (the fine runs have no diffusion)
        valid = [k for k in range(members) if np.all(np.isfinite(ref[k][s][0])) and np.all(np.isfinite(ref[k][s][1]))]
        truth_members.append(len(valid))
        for name, r in runs.items():
            t, _, _, _ = r.time_steps(n_m if name == "plain_finer" else n_c, total=True, flux=False)
            ms[name] += t
            st = _member_states(r, members)
            if name == "plain_finer":
                st = [cg_mc(gd=gd, u=u)[:2] for gd, u in st]
            eh = np.array([_rel_l2(st[k][0], ref[k][s][0], wa) for k in valid])
            eu = np.array([_rel_l2(st[k][1], ref[k][s][1], we) for k in valid])
            fin = np.isfinite(eh) & np.isfinite(eu)
            err[name]["h"].append(float(np.mean(eh[fin])) if fin.any() else float("nan"))
            err[name]["u"].append(float(np.mean(eu[fin])) if fin.any() else float("nan"))
            err[name]["nonfinite"].append(int(np.sum(~fin)))
        if log:
            log(f"day {(s + 1) * total / samples / DAY:.2f}: " +
                ", ".join(f"{n} h {err[n]['h'][-1]:.3e} u {err[n]['u'][-1]:.3e}" for n in runs))
    timed_out = any(runs[name].closure_status() for name in nets)
    for r in runs.values():
        r.close()
    for c in (cg_c, cg_m, cg_mc):
        c.close()
    return {
        "fine_level": fine_level, "coarse_level": coarse_level, "members": members, "days": days,
        "truth": "FP64 runs" if truth_is_fp64 else "FP32 ensemble", "apvm_weight": apvm_weight,
        "truth_fp32_vs_fp64": ({"members": min(truth_check, members),
                                "h_rel_l2_max": [float(max(v)) for v in check["h"]],
                                "u_rel_l2_max": [float(max(v)) for v in check["u"]]}
                               if check["h"][0] else None),
        "times_days": [(s + 1) * total / samples / DAY for s in range(samples)],
        "truth_members": truth_members,
        "error": err,
        "device_s_per_day": {n: ms[n] / 1e3 / days for n in runs},
        "closure_timed_out": timed_out,
    }


class FallbackMonitor:
    """Per-member invariant-drift fallback: every `every` steps, a member whose
    relative drift of total energy (or mass) since its start exceeds `tol`
    gets the closure switched off and its state rolled back to its last
    checkpoint (taken at the previous check)."""

    def __init__(self, model: TMCoreGPU, members: int, tol: float = 1e-3, every: int = 24):
        self.model, self.members, self.tol, self.every = model, members, tol, every
        d = model.diag_all()
        self.ref = d[:, :2].copy()
        self.on = np.ones(members, bool)
        self.fallbacks: list[tuple[int, int]] = []
        self.max_drift = np.zeros(members)  # largest relative energy/mass drift seen per member
        self.steps = 0
        self.ckpt = [self._save(m) for m in range(members)]

    def _save(self, m):
        self.model.select_member(m)
        return self.model.get_state(with_u=False)

    def step(self, n: int):
        """Advance all members n steps, checking every `every` steps."""
        while n > 0:
            k = min(n, self.every - self.steps % self.every)
            self.model.step(k)
            self.steps += k
            n -= k
            if self.steps % self.every == 0:
                self.check()

    def check(self):
        d = self.model.diag_all()
        drift = np.abs(d[:, :2] - self.ref) / np.abs(self.ref)
        self.max_drift = np.maximum(self.max_drift, np.where(np.isfinite(drift.max(1)), drift.max(1), np.inf))
        bad = np.flatnonzero(self.on & ((drift.max(1) > self.tol) | ~np.all(np.isfinite(d[:, :2]), 1)))
        for m in bad:
            self.model.set_member_closure(int(m), False)
            self.on[m] = False
            self.model.select_member(int(m))
            gd, iap = self.ckpt[m]
            self.model.set_state(gd, iap)
            self.fallbacks.append((int(m), self.steps))
        for m in np.flatnonzero(self.on):
            self.ckpt[m] = self._save(int(m))
        return bad


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--fine-level", type=int, default=8)
    ap.add_argument("--coarse-level", type=int, default=6)
    ap.add_argument("--runs", type=int, default=4)
    ap.add_argument("--days", type=float, default=1.0)
    ap.add_argument("--samples", type=int, default=8)
    ap.add_argument("--steps", type=int, default=1500)
    ap.add_argument("--members", type=int, default=256)
    ap.add_argument("--ens-days", type=float, default=1.0)
    ap.add_argument("--every-stage", action="store_true",
                    help="run the network in every stage (default: stage 1, its output held for stages 2-4)")
    ap.add_argument("--eval-members", type=int, default=16, help="held-out seeds of the comparison (0: skip)")
    ap.add_argument("--eval-days", type=float, default=5.0)
    ap.add_argument("--eval-samples", type=int, default=5, help="scoring times of the comparison")
    ap.add_argument("--truth", choices=("fp64", "fp32"), default="fp64",
                    help="the comparison's fine-mesh truth: FP64 runs, or one FP32 ensemble")
    ap.add_argument("--apvm-weight", type=float, default=0.5,
                    help="the comparison's fixed-weight APVM baseline (0: none)")
    ap.add_argument("--truth-check", type=int, default=0,
                    help="with --truth fp32: members also run in FP64 to measure the truths' difference")
    ap.add_argument("--out", default=None, help="save the trained networks (.npz; the head is appended)")
    ap.add_argument("--load", default=None,
                    help="networks saved by --out, comma separated: use them instead of training")
    ap.add_argument("--trainer", choices=("tc", "cuda"), default="tc",
                    help="gradients on the tensor cores (tc) or on the CUDA cores in FP32 (cuda)")
    ap.add_argument("--heads", default="2",
                    help="output heads to train on the same data, comma separated: 1 a learned non-negative "
                         "APVM weight, 2 the residual where it has APVM's sign (both enstrophy-dissipating), "
                         "0 the residual itself")
    ap.add_argument("--train-truth", choices=("fp64", "fp32"), default="fp64",
                    help="the training runs: FP64 one at a time, or one FP32 ensemble of all runs")
    ap.add_argument("--edge-frac", type=float, default=1.0,
                    help="fraction of each training sample's coarse edges kept (random subset)")
    ap.add_argument("--plain-ensemble", action="store_true",
                    help="also run the held-out ensemble without a network, under the same drift monitor")
    a = ap.parse_args()
    say = lambda t: print(t, file=sys.stderr, flush=True)  # noqa: E731
    heads = [int(h) for h in a.heads.split(",") if h != ""]
    dt = level_dt(a.coarse_level)
    nets, losses, t_train = {}, {}, {}
    t_data, n_samples, skipped = 0.0, 0, []
    if a.load:
        heads = []
        for path in a.load.split(","):
            net = load(path)
            nets[net.head] = net
            heads.append(net.head)
    elif heads:
        t0 = time.time()
        X, Y = training_data(a.fine_level, a.coarse_level, a.runs, a.days, a.samples, log=say,
                             truth=a.train_truth, edge_frac=a.edge_frac, skipped=skipped)
        t_data = time.time() - t0
        n_samples = int(len(Y))
        for h in heads:
            t0 = time.time()
            net, ls, sc = train(X, Y, steps=a.steps, tensor_cores=a.trainer == "tc", head=h, dt=dt)
            t_train[h] = time.time() - t0
            nets[h], losses[h] = net, ls
            if a.out:
                save(a.out.replace(".npz", "") + f"_head{h}.npz", net, sc)
            say(f"head {h}: loss {float(ls[0]):.4f} -> {float(np.mean(ls[-20:])):.4f} in {t_train[h]:.1f} s")
        X = Y = None
    # held-out ensembles on the coarse mesh with the closure and the fallback
    coarse = icos_mesh(a.coarse_level)
    ensembles = {}
    for key, net in ([("plain", None)] if a.plain_ensemble else []) + [(f"head{h}", nets[h]) for h in heads]:
        ens = TMCoreGPU(coarse, members=a.members, dt=dt, precision=abi.TMC_FP32, pv_scheme=1, apvm_weight=0.0,
                        diag_every=0, member_layout=1 if a.members % 16 == 0 else 0)
        for m in range(a.members):
            gd, u, ghs = cases.jet_bumps(coarse, seed=10_000 + m)
            ens.select_member(m)
            ens.set_initial(gd, u, ghs)
        if net is not None:
            ens.set_closure(net)
            ens.set_closure_stages(a.every_stage)
        mon = FallbackMonitor(ens, a.members)
        nsteps = int(round(a.ens_days * DAY / dt))
        t0 = time.time()
        mon.step(nsteps)
        ens.synchronize()
        t_ens = time.time() - t0
        kept = mon.on
        ensembles[key] = {
            "members": a.members, "level": a.coarse_level, "steps": nsteps, "wall_s": t_ens,
            "member_days_per_s": a.members * nsteps * dt / DAY / t_ens, "closure": net is not None,
            "every_stage": a.every_stage, "fallbacks": len(mon.fallbacks),
            "fallback_members": len({m for m, _ in mon.fallbacks}), "drift_limit": mon.tol,
            "max_rel_drift": {"max_kept": float(mon.max_drift[kept].max()) if kept.any() else None,
                              "median_kept": float(np.median(mon.max_drift[kept])) if kept.any() else None,
                              "max_all": float(mon.max_drift.max())},
            "closure_timed_out": ens.closure_status()}
        ens.close()
        say(f"ensemble {key}: {ensembles[key]['fallback_members']} members fell back, {t_ens:.1f} s")
    comparison = None
    if a.eval_members > 0 and nets:
        comparison = evaluate({f"closure_head{h}": n for h, n in nets.items()}, a.fine_level, a.coarse_level,
                              members=a.eval_members, days=a.eval_days, samples=a.eval_samples, truth=a.truth,
                              apvm_weight=a.apvm_weight, truth_check=a.truth_check, log=say)
    for n in nets.values():
        n.close()
    print(json.dumps({
        "training_samples": n_samples, "data_s": t_data, "skipped_samples": len(skipped),
        "skipped_runs": sorted({r for r, _ in skipped}), "train_s": t_train, "trainer": a.trainer,
        "heads": heads, "loss_first": {h: float(l[0]) for h, l in losses.items()},
        "loss_last": {h: float(np.mean(l[-20:])) for h, l in losses.items()},
        "ensembles": ensembles, "comparison": comparison,
    }))


if __name__ == "__main__":
    main()
