#!/usr/bin/env python3
"""Benchmark: simulated days per wall-second of the TRiSK shallow-water CRK4
step on one GB300, on the level-9 icosahedral mesh (2,621,442 cells,
7,864,320 edges, 5,242,880 vertices) with 4 coupled tracers and dt = 45 s.

One "step" is one CRK4 time step (4 spatial_operators stages + the beta-scaled
update) of the whole mesh.  The headline arm is the FP32-state path (FP64
metrics, gd accumulation and invariant sums); the plain FP64 path is timed on
the same initial state and the FP32 h error against it is reported.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU FP64 restatement of the reference (the
oracle; the Fortran reference cannot be compiled in this image) on the host
cores, on the same workload.  For N > 1 (torchrun) the path runs as
independent replicas, one per GPU ("replicas only": a single mesh is not
domain-decomposed); the time is the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

DAY = 86400.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--level", type=int, default=9)
    ap.add_argument("--dt", type=float, default=45.0)
    ap.add_argument("--tracers", type=int, default=4)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison run")
    ap.add_argument("--error-days", type=float, default=1.0,
                    help="simulated days of the FP32-vs-FP64 per-field error comparison (0: skip)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-steps", type=int, default=20,
                    help="CRK4 steps of the CPU baseline (stops early past 25 s)")
    ap.add_argument("--no-autotune", action="store_true", help="keep 256-thread blocks")
    ap.add_argument("--ensemble-members", type=int, default=512,
                    help="FP32 ensemble on --ensemble-level (0: skip)")
    ap.add_argument("--ensemble-level", type=int, default=6)
    ap.add_argument("--ensemble-steps", type=int, default=20)
    ap.add_argument("--mixed-members", type=int, default=16, help="members per level of the mixed batch (0: skip)")
    ap.add_argument("--closure-members", type=int, default=256, help="ensemble with the learned closure (0: skip)")
    ap.add_argument("--mixed-cycles", type=int, default=5)
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def job_value(world: int, steps: int, dt: float, ms_max: float) -> float:
    """Whole-job simulated days per wall-second: the days all `world` replicas
    advanced (`steps` steps of `dt` s each) over the slowest rank's time."""
    return world * steps * dt / DAY / (ms_max / 1e3)


class Dist:
    def __init__(self, world):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as td

            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        time.sleep(0.3)

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, smax, pw, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
                pw.append(float(r[3]))
            except (ValueError, IndexError):
                continue
            for k, n in enumerate(names):
                if len(r) > 5 + k and r[5 + k].strip() == "Active":
                    reasons.add(n)
        busy = [s for s in sm if smax and s > 0.5 * max(smax)] or sm
        return {"sm_mhz": statistics.median(busy) if busy else None, "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(pw) if pw else None, "samples": len(sm), "reasons": sorted(reasons)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# Algorithmic (compulsory) bytes of the device kernels: every array read once
# per launch, gathered neighbour values counted once (perfect reuse), writes
# once.  S: bytes of an edge/vertex/tracer state value (4 FP32 path, 8 FP64
# path); Mw: bytes of a metric in the arithmetic (FP32 copies in the FP32
# path, FP64 otherwise); gd is FP64 in both paths.  The layouts are those of
# tmcore_gb300/csrc (structure of arrays, int32 indices, int8 signs).
# ---------------------------------------------------------------------------
def flux_kernel_bytes(nc: int, ne: int, S: int, mode: int | None = None) -> float:
    """k_edge_flux: edgesOnEdge 40, weightsOnEdge 10 Mw, cellsOnEdge 8, dcEdge Mw;
    pv_e, u, F (FP32) or gd_edge (FP64) and own gd_edge: 4 S; RK traffic by
    stage (1: old r, acc/tend/next w; 2,3: areaEdge, tend r+w, acc r+w, old r,
    next w; 4: areaEdge, tend r+w, acc r+w); per cell E (S) and the gd
    tendency (S in the FP32 path's shadow, 8 in FP64)."""
    Mw = S
    rk = {1: 4 * S, 2: Mw + 6 * S, 3: Mw + 6 * S, 4: Mw + 4 * S}
    modes = [mode] if mode else [1, 2, 3, 4]
    tot = 0.0
    for md in modes:
        tot += ne * (40 + 10 * Mw + 8 + Mw + 4 * S + rk[md]) + nc * (S + S)
        if md <= 3:
            # fused preparation of the next stage: next gd gathered, gd_edge/u/F
            # written instead of the next stage's iap_u
            tot += nc * S + ne * 2 * S
    return tot / len(modes)


def pass_bytes(nc: int, ne: int, nv: int, S: int, ntr: int, diag: bool = True) -> dict:
    """Algorithmic bytes of each pass of one CRK4 step (4 stages of cell,
    vertex, edge_pv, edge_flux with the invariants on stage 1; stages 1-3 of
    the flux pass also prepare the next stage's gd_edge, u, F), then the final
    update of cells and of edges (which prepares the next step's first stage),
    as mean bytes per launch."""
    Mw = S
    sh = 4 if S == 4 else 0  # FP32 shadows
    cell = vert = epv = flux = 0.0
    for k in (1, 2, 3, 4):
        dg = diag and k == 1
        # cell, access by access; per edge u, F, dvEdge, areaEdge (16 B FP32); the neighbours'
        # tracer values come from the same array as the cell's own (perfect reuse)
        if S == 4:
            # k_cell_fast: edgesOnCell, nSign, cellsOnCell (tracers), 1/areaCell (f64 and f32), the
            # gd and ghs shadows, E out; RK of gd: old r (stages 1-3), acc r (2-4) and w, tendency
            # shadow r (2-4) and w, areaCell_f (2-4), next gd and its shadow w (1-3); per tracer:
            # ratio r, mass of old r (1-3), acc r (2-4) and w, next ratio w (1-3); invariants
            # (stage 1): gd, areaCell, areaCell_f
            base = 24 + 6 + (24 if ntr else 0) + 8 + 4 + 4 + 4 + 4
            rk_gd = {1: 32, 2: 48, 3: 48, 4: 28}[k]
            trq = {1: 16, 2: 20, 3: 20, 4: 12}[k]
            dgb = 20
        else:
            # k_cell<double>: nEdgesOnCell, edgesOnCell, nSign, cellsOnCell (tracers), areaCell, gd,
            # ghs, E out; RK of gd; per tracer: mass of the stage r (= old in stage 1), old r
            # (2-3), acc r (2-4) and w, next w (1-3)
            base = 1 + 24 + 6 + (24 if ntr else 0) + 8 + 3 * 8
            rk_gd = {1: 32, 2: 48, 3: 48, 4: 32}[k]
            trq = {1: 24, 2: 40, 3: 40, 4: 24}[k]
            dgb = 24
        cell += nc * (base + rk_gd + ntr * trq + (dgb if dg else 0)) + ne * (2 * S + 2 * Mw)
        # vertex: cellsOnVertex, edgesOnVertex, kite, tSign, 1/areaTriangle, fVertex; pv out;
        # gd and u, dcEdge gathered
        vert += nv * (12 + 12 + 3 * Mw + 3 + Mw + Mw + S + (16 if dg else 0)) + nc * S + ne * (S + Mw)
        # edge_pv: verticesOnEdge; pv_e out; pv gathered
        epv += ne * (8 + S) + nv * S
        flux += flux_kernel_bytes(nc, ne, S, k)
    # final cells: gd r+w, acc r, shadow w; tracers r+w, acc r, shadow w
    # final edges: iap_u r+w, acc r, cellsOnEdge, gd gathered, gd_edge/u/F written, areaEdge (energy)
    final = nc * (24 + sh + ntr * (3 * S + sh)) + ne * (3 * S + 8 + 3 * S + Mw) + nc * S
    return {"cell": cell / 4, "vertex": vert / 4, "edge_pv": epv / 4, "edge_flux": flux / 4, "final": final}


def step_bytes(nc: int, ne: int, nv: int, S: int, ntr: int, diag: bool = True) -> float:
    """All kernels of one CRK4 step (pass_bytes: four launches of each stage
    pass and one final update)."""
    b = pass_bytes(nc, ne, nv, S, ntr, diag)
    return 4 * (b["cell"] + b["vertex"] + b["edge_pv"] + b["edge_flux"]) + b["final"]


def step_model_bytes(nc: int, ne: int, nv: int, S: int, ntr: int) -> float:
    """The hot-path scope's per-step compulsory-traffic model (FP64 metrics,
    each mesh array read once per stage, state read/written once per stage;
    4 stages + the final update), plus the coupled tracers in FP64."""
    per_stage = 39 * nc + 153 * ne + 67 * nv + 8 * S * nc + 7 * S * ne
    tracer_stage = ntr * (5 * 8 * nc + 2 * S * ne)
    return 4 * (per_stage + tracer_stage) + 3 * S * (nc + ne) + ntr * 3 * 8 * nc


def ensemble_model_bytes(nc: int, ne: int, nv: int, S: int, members: int) -> float:
    """The hot-path scope's per-step model with `members` models sharing one
    mesh: mesh arrays once per stage, state per member."""
    return 4 * (39 * nc + 153 * ne + 67 * nv + members * (8 * S * nc + 7 * S * ne)) + 3 * S * members * (nc + ne)


def inner_ensemble_pass_bytes(nc: int, ne: int, nv: int, members: int) -> dict:
    """Algorithmic bytes per launch of each pass of the member-innermost
    ensemble step (every array once per pass, gathers at perfect reuse),
    averaged over the four CRK4 stages: FP32 edge and vertex fields, gd and
    its RK accumulator double-float (8 bytes), mesh tables once per pass.
    Per member and stage (modes 1 / 2-3 / 4):
      cell   u, F 8 Ne; gd old 8, acc 8 / 16 / 8, tend 0 / 4 / 4 in, gd h, ghs 8,
             E 4, acc 8, tend 4, next gd 8 / 8 / 0 out  (+4 Nc gd l on the diag stage)
      vertex gd h 4 Nc, u 4 Ne in, pv 4 Nv out
      edge_pv pv 4 Nv in, pv_e 4 Ne out
      flux   pv_e, u, gd_e, F 16, tend + acc 0 / 8 / 8, old 4 / 4 / 0, acc + tend 8,
             next gd_e, u, F 12 / 12 / 0 per edge; E, tend, next gd h 12 / 12 / 8 per cell
      final  cells gd r/w 16, acc 8; edges iap r/w 8, acc 4, gd_e, u, F 12, gd h 4 Nc."""
    M = members
    mesh = {"cell": 39 * nc + 8 * ne, "vertex": 67 * nv, "edge_pv": 8 * ne, "edge_flux": 153 * ne, "final": 8 * ne}
    per = {
        "cell": (32 * ne + 184 * nc + 4 * nc) / 4.0,
        "vertex": 4 * nc + 4 * ne + 4 * nv,
        "edge_pv": 4 * nv + 4 * ne,
        "edge_flux": (168 * ne + 44 * nc) / 4.0,
        "final": 28 * nc + 24 * ne,
    }
    return {k: mesh[k] + M * per[k] for k in per}


def inner_ensemble_step_bytes(nc: int, ne: int, nv: int, members: int) -> float:
    b = inner_ensemble_pass_bytes(nc, ne, nv, members)
    return 4 * (b["cell"] + b["vertex"] + b["edge_pv"] + b["edge_flux"]) + b["final"]


def _ensemble_ic(job):
    """Initial state of one ensemble member (runs in a spawned worker)."""
    level, seed = job
    from tmcore_gb300 import cases, mesh

    return cases.jet_bumps(mesh.icos_mesh(level), seed=seed)


def ensemble_ics(level: int, members: int, mixed_levels=(), mixed_members: int = 0):
    """Seeds 0..members-1 on `level`, and seeds 0..mixed_members-1 on each of
    `mixed_levels`, generated by a spawn pool (started before any CUDA work)."""
    import multiprocessing as mp

    jobs = [(level, s) for s in range(members)] + [(L, s) for L in mixed_levels for s in range(mixed_members)]
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
        out = pool.map(_ensemble_ic, jobs, chunksize=4)
    mixed = {L: out[members + i * mixed_members: members + (i + 1) * mixed_members]
             for i, L in enumerate(mixed_levels)}
    return out[:members], mixed


def run_mixed(args, local, ics_by_level, peak):
    """Config 3, mixed batch: ensembles on mesh levels 4-7 with dt = 1200 / 2^(L-4) s,
    advanced together as one CUDA graph per 1200-s cycle (tmc_group).  Both member
    layouts are timed when every level's member count is a multiple of 16; the
    faster is reported, the other beside it.  In the member-innermost layout the
    batch takes the lane layout (tune.lane_candidates, one for all levels, so that
    both group schedules apply) whose slowest level, timed alone for its steps of
    a cycle after tuning the block sizes, is fastest."""
    from tmcore_gb300 import abi, mesh, tune
    from tmcore_gb300.gpu import TMCError, TMCoreGPU, TMCoreGroup

    inner_ok = all(len(ics) % 16 == 0 for ics in ics_by_level.values())
    res = {}
    for layout in ((1, 0) if inner_ok else (0,)):
        # lane layouts every level's member count allows
        lanes_ok = [ln for ln in tune.LANES
                    if all(ln in tune.lane_candidates(len(ics)) for ics in ics_by_level.values())] if layout == 1 else [0]
        best, lanes_ms = None, {}  # best: (slowest level's ms per cycle, member_lanes, models)
        for ln in lanes_ok:
            cand, t_lv = [], {}
            for L, ics in sorted(ics_by_level.items()):
                m = mesh.icos_mesh(L)
                dt = 1200.0 / 2 ** (L - 4)
                c = TMCoreGPU(m, members=len(ics), dt=dt, pv_scheme=1, apvm_weight=0.0, adv_order=2,
                              conserve_energy=1, precision=abi.TMC_FP32, diag_every=0, use_graph=1, renumber=1,
                              device=local, member_layout=layout, member_lanes=ln)
                for k, (gd, u, ghs) in enumerate(ics):
                    c.select_member(k)
                    c.set_initial(gd, u, ghs)
                if not args.no_autotune:
                    c.autotune(steps=2)
                if len(lanes_ok) > 1:  # the level's steps of two cycles, alone
                    ms, _, _, _ = c.time_steps(2 ** (L - 3), total=True, flux=False)
                    t_lv[f"L{L}"] = ms / 2
                cand.append(c)
            worst = max(t_lv.values()) if t_lv else 0.0
            lanes_ms[str(ln)] = t_lv
            if best is None or worst < best[0]:
                if best is not None:
                    for c in best[2]:
                        c.close()
                best = (worst, ln, cand)
            else:
                for c in cand:
                    c.close()
        models, bytes_cycle, members, desc = best[2], 0.0, 0, []
        for (L, ics), e in zip(sorted(ics_by_level.items()), models):
            m = mesh.icos_mesh(L)
            dt = 1200.0 / 2 ** (L - 4)
            members += len(ics)
            bytes_cycle += (1200.0 / dt) * ensemble_model_bytes(m.nCells, m.nEdges, m.nVertices, 4, len(ics))
            desc.append(f"L{L}x{len(ics)} dt={dt:g}s")
        lanes_ms = {"member_lanes": best[1], "ms_per_cycle_by_lanes_and_level": lanes_ms} if layout == 1 else {}
        cycles = args.mixed_cycles
        by_mode = {}
        for mode in ((0, 1) if layout == 1 else (0,)):
            # mode 0: one graph branch per level; mode 1: one launch per pass over all levels
            # (it refuses levels whose lane layouts differ)
            try:
                grp = TMCoreGroup(models, cycle_seconds=1200.0, mode=mode)
            except TMCError:
                continue
            grp.run(1)
            grp.synchronize()
            t = time.perf_counter()
            grp.run(cycles)
            grp.synchronize()
            by_mode[mode] = (time.perf_counter() - t) / cycles
            grp.close()
        group_mode = min(by_mode, key=by_mode.get)
        el = by_mode[group_mode] * cycles
        # each level alone: its steps of one cycle (CUDA events) and its passes
        alone = {}
        for L, e in zip(sorted(ics_by_level), models):
            n = 2 ** (L - 4)  # steps per 1200-s cycle
            ms, _, _, _ = e.time_steps(2 * n, total=True, flux=False)
            alone[f"L{L}"] = {"ms_per_cycle": ms / 2, "passes_ms": e.pass_times(2)}
            e.close()
        res[layout] = (el / cycles, members, desc, bytes_cycle, alone, group_mode, by_mode, lanes_ms)
    lay = min(res, key=lambda k: res[k][0])  # the faster layout
    cyc_s, members, desc, bytes_cycle, alone, group_mode, by_mode, lanes_ms = res[lay]
    pm = sum(2 ** (L - 4) * inner_ensemble_step_bytes(10 * 4 ** L + 2, 30 * 4 ** L,
                                                                              20 * 4 ** L, len(ics))
             for L, ics in ics_by_level.items())
    out = {"workload": "mixed batch " + ", ".join(desc) + ", one CUDA graph per 1200-s cycle",
           "member_layout": lay, "group_mode": group_mode,
           "group_mode_ms_per_cycle": {("one launch per pass over all levels" if k == 1 else "a graph branch per level"):
                                       v * 1e3 for k, v in by_mode.items()},
           "members": members, "cycles": args.mixed_cycles, "ms_per_cycle": cyc_s * 1e3,
           "member_days_per_s": members * 1200.0 / DAY / cyc_s, "sim_days_per_s": 1200.0 / DAY / cyc_s,
           "scope_model_bytes_per_cycle": bytes_cycle, "achieved_gbs": bytes_cycle / cyc_s / 1e9,
           "frac": bytes_cycle / cyc_s / 1e9 / peak, "pass_model_bytes_per_cycle": pm,
           "pass_model_frac": pm / cyc_s / 1e9 / peak, "levels_alone": alone, "member_lanes_by_level": lanes_ms,
           "timing": "host wall clock around tmc_group_run + sync; levels alone: CUDA events"}
    for other in res:
        if other != lay:
            c0 = res[other][0]
            out["other_layout"] = {"member_layout": other, "ms_per_cycle": c0 * 1e3,
                                   "member_days_per_s": members * 1200.0 / DAY / c0}
    return out


def run_ensemble(args, local, ics, peak):
    """Config 3: FP32 members of one mesh stepped together, CUDA graph per CRK4
    step; dt = 1200 / 2^(level-4) s.  Member-innermost layout (member_layout 1:
    arrays [element][member], a warp per 32 members of an element), with the
    member-outermost layout (member = blockIdx.y) timed beside it."""
    from tmcore_gb300 import abi, mesh
    from tmcore_gb300.gpu import TMCoreGPU

    L, M = args.ensemble_level, len(ics)
    m = mesh.icos_mesh(L)
    dt = 1200.0 / 2 ** (L - 4)

    def timed(layout, **scheme):
        ens = TMCoreGPU(m, members=M, dt=dt, adv_order=2, conserve_energy=1, precision=abi.TMC_FP32, diag_every=1,
                        use_graph=1, renumber=1, device=local, member_layout=layout, **scheme)
        for k, (gd, u, ghs) in enumerate(ics):
            ens.select_member(k)
            ens.set_initial(gd, u, ghs)
        tuned = ens.autotune(steps=2) if not args.no_autotune else None
        ens.step(args.warmup)
        ens.synchronize()
        ms, _, _, launches = ens.time_steps(args.ensemble_steps, total=True, flux=False)
        passes = ens.pass_times(3) if layout == 1 else None
        d = ens.diag()
        ens.close()
        return ms / args.ensemble_steps / 1e3, launches, d, tuned, passes

    centred = dict(pv_scheme=1, apvm_weight=0.0)
    res = {layout: timed(layout, **centred) for layout in ((1, 0) if M % 32 == 0 else (0,))}
    lay = 1 if 1 in res else 0
    step_s, launches, d, tuned, passes = res[lay]
    mb = ensemble_model_bytes(m.nCells, m.nEdges, m.nVertices, 4, M)
    out = {"workload": f"{M} FP32 members on level {L} ({m.nCells} cells), seeds 0..{M - 1}, CRK4 dt={dt:g}s",
           "member_layout": lay, "members": M, "level": L, "dt_s": dt, "steps": args.ensemble_steps,
           "ms_per_step": step_s * 1e3, "member_days_per_s": M * dt / DAY / step_s, "sim_days_per_s": dt / DAY / step_s,
           "scope_model_bytes_per_step": mb, "achieved_gbs": mb / step_s / 1e9, "frac": mb / step_s / 1e9 / peak,
           "gpu_launches": launches, "member0_beta": float(d[4]), "block_sizes": tuned}
    if lay == 1:
        pb = inner_ensemble_pass_bytes(m.nCells, m.nEdges, m.nVertices, M)
        sb = inner_ensemble_step_bytes(m.nCells, m.nEdges, m.nVertices, M)
        out["pass_model_bytes_per_step"] = sb
        out["pass_model_frac"] = sb / step_s / 1e9 / peak
        out["passes"] = {k: {"ms_per_launch": passes[k], "algorithmic_bytes_per_launch": pb[k],
                             "achieved_gbs": pb[k] / (passes[k] * 1e-3) / 1e9,
                             "frac": pb[k] / (passes[k] * 1e-3) / 1e9 / peak} for k in pb}
    if 0 in res and lay == 1:
        s0 = res[0][0]
        out["member_outermost"] = {"ms_per_step": s0 * 1e3, "member_days_per_s": M * dt / DAY / s0,
                                   "block_sizes": res[0][3]}
    if lay == 1:
        # the reference namelist's pv scheme: upwind pv on edges, interp_pv_order 3
        up = {k: timed(k, pv_scheme=3, interp_pv_order=3) for k in (1, 0)}
        out["upwind_pv"] = {"pv_scheme": 3, "interp_pv_order": 3,
                            "ms_per_step": up[1][0] * 1e3, "member_days_per_s": M * dt / DAY / up[1][0],
                            "edge_pv_ms_per_launch": up[1][4]["edge_pv"],
                            "member_outermost_ms_per_step": up[0][0] * 1e3}
    return out


def run_closure_leg(args, local, ics, peak):
    """Config 5's step: the FP32 ensemble with the learned closure on (a
    network of the trained shape with the APVM head; the cost does not depend
    on its weights) in
    every stage and in stage 1 only (held for stages 2-4), against the same
    ensemble without it; member-outermost layout, and the member-innermost
    layout beside it when the member count allows."""
    import numpy as np

    from tmcore_gb300 import abi, mesh
    from tmcore_gb300.gpu import ClosureMLP, TMCoreGPU

    L, M = args.ensemble_level, len(ics)
    m = mesh.icos_mesh(L)
    dt = 1200.0 / 2 ** (L - 4)
    net = ClosureMLP(device=local, seed=1)
    res = {}
    for layout in ((0, 1) if M % 16 == 0 else (0,)):
        ens = TMCoreGPU(m, members=M, dt=dt, pv_scheme=1, apvm_weight=0.0, adv_order=2, conserve_energy=1,
                        precision=abi.TMC_FP32, diag_every=1, use_graph=1, renumber=1, device=local,
                        member_layout=layout)
        for k, (gd, u, ghs) in enumerate(ics):
            ens.select_member(k)
            ens.set_initial(gd, u, ghs)
        if not args.no_autotune:
            ens.autotune(steps=2)
        ens.step(args.warmup)
        ens.synchronize()
        ms_plain, _, _, _ = ens.time_steps(args.ensemble_steps, total=True, flux=False)
        if layout == 0:
            # the shipped form: the APVM head (a learned non-negative APVM
            # weight), inputs normalised by one member's feature statistics
            feats, _ = ens.closure_features()
            sd = feats.std(0).astype(np.float64)
            sd[sd == 0] = 1.0
            net.set_scaling(feats.mean(0), 1.0 / sd, 1.0)
            net.set_head(1, dt)
        ens.set_closure(net)
        ens.step(args.warmup)
        ens.synchronize()
        ms, _, _, launches = ens.time_steps(args.ensemble_steps, total=True, flux=False)
        ens.set_closure_stages(False)  # the network in stage 1, its output held for stages 2-4
        ens.step(args.warmup)
        ens.synchronize()
        ms_s1, _, _, _ = ens.time_steps(args.ensemble_steps, total=True, flux=False)
        timed_out = ens.closure_status()
        ens.close()
        K = args.ensemble_steps
        res[layout] = (ms / K, ms_plain / K, ms_s1 / K, launches, timed_out)
    net.close()
    head = 1 if 1 in res else 0  # the member-innermost step is the faster when it applies
    ms, ms_plain, ms_s1, launches, timed_out = res[head]
    step_s = ms / 1e3
    flops = 4 * M * m.nEdges * 2.0 * (32 * 64 + 2 * 64 * 64)  # tensor-core MMA flops per step (K padded to 32)
    out = {"workload": f"{M} FP32 members on level {L} with the learned PV-on-edge closure every stage",
           "member_layout": head, "members": M, "ms_per_step": ms, "member_days_per_s": M * dt / DAY / step_s,
           "plain_ms_per_step": ms_plain, "stage1_ms_per_step": ms_s1,
           "stage1_member_days_per_s": M * dt / DAY / (ms_s1 / 1e3),
           "closure_tflops": flops / 1e12 / (step_s - ms_plain / 1e3) if ms > ms_plain else None,
           "closure_mma_tflops_per_step": flops / 1e12, "gpu_launches": launches, "timed_out": timed_out}
    for other in res:
        if other != head:
            ms1, plain1, s11, _, to1 = res[other]
            out["other_layout"] = {"member_layout": other, "ms_per_step": ms1, "plain_ms_per_step": plain1,
                                   "stage1_ms_per_step": s11, "member_days_per_s": M * dt / DAY / (ms1 / 1e3),
                                   "stage1_member_days_per_s": M * dt / DAY / (s11 / 1e3), "timed_out": to1}
    return out


def run_training_leg(args, local):
    """Config 4's kernels: Adam steps of the closure network on batches of
    65536 rows (synthetic features and a smooth target of the network's
    input width), with the forward and backward on the tensor cores (the
    headline) and on the CUDA cores in FP32, and the tensor-core forward on
    the same rows.  Host wall clock around the calls, which synchronise; the
    forward includes its host copies (24 + 1 floats per row)."""
    import numpy as np

    from tmcore_gb300.gpu import ClosureMLP

    rows, batch, steps = 1 << 20, 65536, 50
    rng = np.random.default_rng(0)
    x = rng.standard_normal((rows, 24)).astype(np.float32)
    y = (0.3 * np.tanh(x[:, 0] * x[:, 1]) + 0.1 * x[:, 2]).astype(np.float32)
    res = {}
    for tc in (True, False):
        net = ClosureMLP(device=local, seed=3)
        net.set_train_mode(tc)
        net.set_scaling(np.zeros(24), np.ones(24), 1.0)
        net.set_dataset(x, y)
        net.train(5, batch=batch)
        t = time.perf_counter()
        losses = net.train(steps, batch=batch)
        res[tc] = ((time.perf_counter() - t) / steps, losses)
        if tc:
            net.forward(x[:batch])
            t = time.perf_counter()
            net.forward(x)
            fwd_s = time.perf_counter() - t
        net.close()
    train_s, losses = res[True]
    flops_row = 2.0 * (24 * 64 + 2 * 64 * 64 + 64)
    return {"workload": f"closure network 24-64-64-64-1, Adam (lr 1e-3) on batches of {batch} rows, "
                        f"{rows} synthetic rows", "batch": batch, "steps": steps,
            "trainer": "tensor cores (tcgen05 forward and backward, BF16 operands, FP32 accumulation)",
            "ms_per_batch": train_s * 1e3, "train_rows_per_s": batch / train_s,
            "train_tflops": 3 * flops_row * batch / train_s / 1e12,
            "cuda_cores_fp32_ms_per_batch": res[False][0] * 1e3,
            "forward_rows_per_s_with_copies": rows / fwd_s, "loss_first_last": [float(losses[0]), float(losses[-1])],
            "cuda_cores_loss_first_last": [float(res[False][1][0]), float(res[False][1][-1])],
            "timing": "host wall clock around tmc_mlp_train / tmc_mlp_forward (both synchronise)"}


def ncu_traffic(name: str):
    """dram bytes per launch from the committed ncu summary, if present."""
    p = os.path.join(ROOT, "profiles", name)
    if os.path.exists(p):
        try:
            return json.load(open(p)).get("dram_bytes_per_launch")
        except (ValueError, OSError):
            return None
    return None


def setup(args):
    from tmcore_gb300 import cases, mesh

    t0 = time.time()
    m = mesh.generate_icos(args.level, 20)
    gd, u, ghs = cases.jet_bumps(m, seed=args.seed)
    q = cases.smooth_tracers(m, args.tracers, seed=args.seed) if args.tracers else None
    return m, gd, u, ghs, q, time.time() - t0


def gpu_params(args, precision):
    return dict(dt=args.dt, pv_scheme=1, apvm_weight=0.0, adv_order=2, conserve_energy=1,
                n_tracers=args.tracers, precision=precision, diag_every=1, use_graph=1, renumber=1)


def cpu_baseline(m, gd, u, ghs, q, args, steps: int, threads: int):
    """Time the CPU FP64 oracle (restatement of the reference) on the same workload."""
    from oracle.oracle import Oracle

    o = Oracle(m, dt=args.dt, pv_scheme=1, apvm_weight=0.0, adv_order=2, n_tracers=args.tracers, nthreads=threads)
    o.set_initial(gd, u, ghs)
    if args.tracers:
        o.set_tracers(q * gd[None, :])
    # a bounded sample: `steps` steps, stopping early once 25 s have passed
    t0 = time.perf_counter()
    done = 0
    while done < steps:
        o.step(1)
        done += 1
        if time.perf_counter() - t0 > 25.0:
            break
    dt = time.perf_counter() - t0
    o.close()
    return done * args.dt / DAY / dt, dt, done


def run_reference(args, rank, world):
    """--impl reference: the oracle port on all host cores, same metric and config."""
    if rank != 0:
        return
    m, gd, u, ghs, q, _ = setup(args)
    threads = os.cpu_count() or 1
    from oracle.oracle import Oracle

    o = Oracle(m, dt=args.dt, pv_scheme=1, apvm_weight=0.0, adv_order=2, n_tracers=args.tracers, nthreads=threads)
    o.set_initial(gd, u, ghs)
    if args.tracers:
        o.set_tracers(q * gd[None, :])
    o.step(args.warmup)
    # bounded sample: K steps, stopping early once the timed region passes 150 s
    t0 = time.perf_counter()
    done = 0
    while done < args.steps:
        o.step(1)
        done += 1
        if time.perf_counter() - t0 > 150.0:
            break
    el = time.perf_counter() - t0
    o.close()
    v = done * args.dt / DAY / el
    unit = "simulated days/wall-s"
    line = {
        "impl": "reference", "metric": "simulated days/wall-s", "value": v, "unit": unit, "n_gpus": world,
        "steps": done, "steps_requested": args.steps, "warmup": args.warmup, "ms_per_step": el / done * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_dict(args, m),
        "path": "FP64 CPU restatement of the reference (oracle port)",
        "cpu_baseline": {"value": v, "unit": unit, "cores": threads, "kind": "port",
                         "sample": f"{done} CRK4 steps of the level-{args.level} workload"},
        "e2e": {"value": v, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def config_dict(args, m):
    """The workload, identical in both arms (the path that runs it is a key of its own)."""
    return {"workload": f"level-{args.level} icosahedral SCVT sphere ({m.nCells} cells, {m.nEdges} edges, "
                        f"{m.nVertices} vertices), seeded jet+mountains, {args.tracers} tracers, CRK4 dt={args.dt:g}s",
            "level": args.level, "nCells": m.nCells, "nEdges": m.nEdges, "nVertices": m.nVertices,
            "dt_s": args.dt, "tracers": args.tracers, "pv_scheme": 1, "apvm_weight": 0.0, "adv_order": 2,
            "conserve_energy": True, "seed": args.seed,
            "l2": "inputs larger than L2 (mesh tables + state > 1 GB per stage)"}


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import numpy as np

    from tmcore_gb300 import abi
    from tmcore_gb300.gpu import TMCoreGPU

    # ensemble initial states from a spawn pool, before any CUDA work
    ens_ics, mixed_ics = None, None
    if args.ensemble_members > 0 or args.mixed_members > 0:
        ens_ics, mixed_ics = ensemble_ics(args.ensemble_level, max(args.ensemble_members, 0),
                                          (4, 5, 6, 7) if args.mixed_members > 0 else (), args.mixed_members)
        if args.ensemble_members <= 0:
            ens_ics = None
    dist = Dist(world)
    args.seed += rank  # independent replicas: rank r starts from seed + r
    m, gd, u, ghs, q, t_setup = setup(args)
    qgd = q * gd[None, :] if args.tracers else None

    gpu = TMCoreGPU(m, **gpu_params(args, abi.TMC_FP32), device=local)
    gpu.set_initial(gd, u, ghs)
    if args.tracers:
        gpu.set_tracers(qgd)
    d0_mass = gpu.diag()[0]
    tuned = gpu.autotune(steps=3) if not args.no_autotune else None
    gpu.step(args.warmup)
    gpu.synchronize()

    # ---- timed region: exactly K steps, CUDA graph per step ----
    clocks = Clocks(local)
    clocks.start()
    dist.barrier()
    gpu.synchronize()
    ms_total, _, _, launches = gpu.time_steps(args.steps, total=True, flux=False)
    dist.barrier()
    clk = clocks.stop()
    ms_max = dist.max(ms_total)
    days = world * args.steps * args.dt / DAY
    value = job_value(world, args.steps, args.dt, ms_max)

    gd32, _, u32 = gpu.get_state()
    d32 = gpu.diag()

    # ---- dominant kernel (edge flux pass), launch by launch with events ----
    _, ms_flux, n_flux, _ = gpu.time_steps(max(2, min(args.steps, 10)), total=False, flux=True)
    S = 4
    fb = flux_kernel_bytes(m.nCells, m.nEdges, S)
    t_launch = ms_flux / n_flux / 1e3
    achieved = fb / t_launch / 1e9
    peak, peak_kind = measured_peaks()
    traffic = ncu_traffic("edge_flux_level9_fp32.json")

    sbytes = step_bytes(m.nCells, m.nEdges, m.nVertices, S, args.tracers)
    # every pass of the step, launch by launch (CUDA events around the pass)
    pt = gpu.pass_times(max(2, min(args.steps, 6)))
    pb = pass_bytes(m.nCells, m.nEdges, m.nVertices, S, args.tracers)
    passes = {k: {"ms_per_launch": pt[k], "algorithmic_bytes_per_launch": pb[k],
                  "achieved_gbs": pb[k] / (pt[k] / 1e3) / 1e9, "frac": pb[k] / (pt[k] / 1e3) / 1e9 / peak}
              for k in pt if pt[k] > 0}
    scope_bytes = step_model_bytes(m.nCells, m.nEdges, m.nVertices, S, args.tracers)
    step_s = ms_total / args.steps / 1e3

    # ---- FP32 h error against the plain FP64 path after the same warmup + K steps ----
    extra = {}
    if not args.no_fp64:
        g64 = TMCoreGPU(m, **gpu_params(args, abi.TMC_FP64), device=local)
        g64.set_initial(gd, u, ghs)
        if args.tracers:
            g64.set_tracers(qgd)
        g64.step(args.warmup)
        g64.synchronize()
        ms64, _, _, _ = g64.time_steps(args.steps, total=True, flux=False)
        gd64, _, u64 = g64.get_state()
        d64 = g64.diag()
        area = m.areaCell
        h32, h64 = gd32 / 9.80616, gd64 / 9.80616
        extra["fp64"] = {
            "value": args.steps * args.dt / DAY / (ms64 / 1e3), "unit": "simulated days/wall-s",
            "ms_per_step": ms64 / args.steps,
            "step_gbs": step_bytes(m.nCells, m.nEdges, m.nVertices, 8, args.tracers) / (ms64 / args.steps / 1e3) / 1e9,
            "bound": "fp64 pipe (GB300 FP64 issue rate is 1/64 of FP32)"}
        extra["h_error_fp32_vs_fp64"] = {
            "rel_max": float(np.max(np.abs(h32 - h64)) / np.max(np.abs(h64))),
            "rel_l2": float(np.sqrt(np.sum(area * (h32 - h64) ** 2) / np.sum(area * h64 ** 2))),
            "u_rel_max": float(np.max(np.abs(u32 - u64)) / np.max(np.abs(u64))),
            "after_steps": args.warmup + args.steps}
        if args.error_days > 0:
            # the FP32 path against the FP64 path after whole simulated days, per field
            n = int(round(args.error_days * DAY / args.dt))
            g64.step(max(0, n - args.warmup - args.steps))
            g32 = TMCoreGPU(m, **gpu_params(args, abi.TMC_FP32), device=local)
            g32.set_initial(gd, u, ghs)
            if args.tracers:
                g32.set_tracers(qgd)
            g32.step(n)
            a32, _, v32 = g32.get_state()
            a64, _, v64 = g64.get_state()
            h32, h64 = a32 / 9.80616, a64 / 9.80616
            el = m.dvEdge * m.dcEdge
            err = {"steps": n, "days": n * args.dt / DAY,
                   "h_rel_max": float(np.max(np.abs(h32 - h64)) / np.max(np.abs(h64))),
                   "h_rel_l2": float(np.sqrt(np.sum(area * (h32 - h64) ** 2) / np.sum(area * h64 ** 2))),
                   "u_rel_max": float(np.max(np.abs(v32 - v64)) / np.max(np.abs(v64))),
                   "u_rel_l2": float(np.sqrt(np.sum(el * (v32 - v64) ** 2) / np.sum(el * v64 ** 2)))}
            if args.tracers:
                q32, q64 = g32.get_tracers() / a32[None, :], g64.get_tracers() / a64[None, :]
                err["tracer_rel_max"] = [float(np.max(np.abs(q32[k] - q64[k])) / np.max(np.abs(q64[k])))
                                         for k in range(args.tracers)]
            err["mass_drift_fp32"] = float((g32.diag()[0] - d0_mass) / d0_mass)
            extra["error_fp32_vs_fp64"] = err
            g32.close()
        g64.close()
    extra["invariants_fp32"] = {"mass": d32[0], "energy": d32[1], "enstrophy": d32[2], "abs_vorticity": d32[3],
                                "beta": d32[4]}

    # ---- e2e: the C-ABI drop-in for time_integrate with page-locked host arrays ----
    e2e = None
    if not args.no_e2e:
        import torch

        nc, ne, nt = m.nCells, m.nEdges, args.tracers
        pin = lambda n: torch.empty(n, dtype=torch.float64).pin_memory().numpy()  # noqa: E731
        gA, iA, gB, iB = pin(nc), pin(ne), pin(nc), pin(ne)
        qA = pin(nt * nc).reshape(nt, nc) if nt else None
        qB = pin(nt * nc).reshape(nt, nc) if nt else None
        g0, i0, _ = gpu.get_state()
        gA[:] = g0
        iA[:] = i0
        if nt:
            qA[:] = gpu.get_tracers()
        gpu.time_integrate(gA, iA, qA, out=(gB, iB, qB))  # warm
        dist.barrier()
        t0 = time.perf_counter()
        for k in range(args.steps):
            if k % 2 == 0:
                gpu.time_integrate(gB, iB, qB, out=(gA, iA, qA))
            else:
                gpu.time_integrate(gA, iA, qA, out=(gB, iB, qB))
        el = dist.max(time.perf_counter() - t0)
        bytes_io = 8 * (nc + ne + nt * nc)
        e2e = {"value": days / el, "unit": "simulated days/wall-s", "h2d_bytes_per_step": bytes_io,
               "d2h_bytes_per_step": bytes_io, "ms_per_step": el / args.steps * 1e3,
               "call": "tmc_time_integrate (host state in, host state out, every step)"}

    if ens_ics is not None:
        extra["ensemble"] = run_ensemble(args, local, ens_ics, peak)
        if args.closure_members > 0:
            extra["closure"] = run_closure_leg(args, local, ens_ics[:args.closure_members], peak)
            extra["training"] = run_training_leg(args, local)
        ens_ics = None
    if mixed_ics:
        extra["mixed_batch"] = run_mixed(args, local, mixed_ics, peak)
        mixed_ics = None

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        v, el, done = cpu_baseline(m, gd, u, ghs, q, args, args.cpu_steps, threads)
        cpu = {"value": v, "unit": "simulated days/wall-s", "cores": threads, "kind": "port",
               "sample": f"{done} CRK4 step(s) of the same level-{args.level} workload, FP64 oracle, "
                         f"{el:.1f} s"}
    gpu.close()
    dist.close()
    if rank != 0:
        return
    line = {
        "metric": "simulated days/wall-s", "value": value, "unit": "simulated days/wall-s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded initial state on a generated mesh)",
        "config": config_dict(args, m),
        "path": "FP32 state + FP64 metrics/gd/sums, CUDA graph per CRK4 step",
        "block_sizes": tuned,
        "clocks": clk,
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": "k_edge_flux<float>", "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "algorithmic_bytes_per_launch": fb, "launch_ms": t_launch * 1e3, "launches_timed": n_flux},
        "passes": passes,
        "step_roofline": {"algorithmic_bytes_per_step": sbytes, "achieved_gbs": sbytes / step_s / 1e9,
                          "frac": sbytes / step_s / 1e9 / peak,
                          "scope_model_bytes_per_step": scope_bytes,
                          "scope_model_frac": scope_bytes / step_s / 1e9 / peak},
        "setup_s": t_setup,
    }
    # the long legs first; the FP64 rate and the FP32-vs-FP64 errors last, so
    # that a log that keeps only the end of the line still holds them
    for k in ("ensemble", "closure", "training", "mixed_batch"):
        if k in extra:
            line[k] = extra.pop(k)
    line["passes"] = line.pop("passes")
    line["step_roofline"] = line.pop("step_roofline")
    line["e2e"] = e2e
    line["cpu_baseline"] = cpu
    for k in ("invariants_fp32", "fp64", "h_error_fp32_vs_fp64", "error_fp32_vs_fp64"):
        if k in extra:
            line[k] = extra.pop(k)
    line.update(extra)
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
