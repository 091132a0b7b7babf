"""TEST INFRASTRUCTURE ONLY: the reference's CPU cost, measured with the FP64
oracle (the C restatement of TMCORE's serial Fortran hot path; the Fortran
itself cannot be built in this image).

For each benchmark configuration the oracle runs on the same mesh, initial
state and time step as the GPU path, single-threaded and with OpenMP over all
host cores (``os.cpu_count()``; the reference's own build asks GCC for 8
auto-parallel threads, CMakeLists.txt:14), and each rate is the median of
three timed samples.  A sample is a bounded number of steps; the rate is
simulated days per wall second (member-days for ensembles), timed with a
monotonic clock around the step calls only (no set-up, no I/O).

  python -m oracle.time_baseline [--repeats 3] [--out result.json]

Configurations:
  level5   10,242 cells, dt 600 s, centred pv: the whole 5-day parity run
           (720 steps) per sample
  level9   2,621,442 cells, 4 tracers, dt 45 s (the roofline run: 1 day)
  ens512   512 members on level 6 (40,962 cells), dt 300 s: members are
           independent, so the ensemble rate is the per-member rate
  mixed    levels 4-7 with 16 members each, dt 1200 / 2^(L-4) s: one
           1200-s cycle is 16 x (1 + 2 + 4 + 8) member-steps
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

DAY = 86400.0


def _timed_steps(m, gd, u, ghs, q, dt, steps, threads):
    from oracle.oracle import Oracle

    ntr = 0 if q is None else q.shape[0]
    o = Oracle(m, dt=dt, pv_scheme=1, apvm_weight=0.0, adv_order=2, n_tracers=ntr, nthreads=threads)
    o.set_initial(gd, u, ghs)
    if ntr:
        o.set_tracers(q * gd[None, :])
    o.step(1)  # warm
    t0 = time.perf_counter()
    o.step(steps)
    el = time.perf_counter() - t0
    o.close()
    return el


def _rate(m, gd, u, ghs, q, dt, steps, threads, repeats):
    els = [_timed_steps(m, gd, u, ghs, q, dt, steps, threads) for _ in range(repeats)]
    el = statistics.median(els)
    return {"steps": steps, "s_median": el, "s_samples": els, "sim_days_per_s": steps * dt / DAY / el,
            "ms_per_step": el / steps * 1e3}


def run(repeats: int = 3, configs=("level5", "level9", "ens512", "mixed"), log=print) -> dict:
    from tmcore_gb300 import cases, mesh

    cores = os.cpu_count() or 1
    out = {"cores_all": cores, "repeats": repeats, "kind": "port", "configs": {}}
    # (level, dt, tracers, single-thread steps, all-core steps)
    plan = {"level5": (5, 600.0, 0, 720, 720), "level9": (9, 45.0, 4, 2, 8), "ens512": (6, 300.0, 0, 16, 64)}
    for name in configs:
        if name in plan:
            L, dt, ntr, s1, sn = plan[name]
            m = mesh.generate_icos(L, 20)
            gd, u, ghs = cases.jet_bumps(m, seed=0)
            q = cases.smooth_tracers(m, ntr, seed=0) if ntr else None
            r1 = _rate(m, gd, u, ghs, q, dt, s1, 1, repeats)
            rn = _rate(m, gd, u, ghs, q, dt, sn, cores, repeats)
            res = {"level": L, "nCells": m.nCells, "dt_s": dt, "tracers": ntr, "single_thread": r1, "all_cores": rn}
            if name == "ens512":
                for r in (r1, rn):
                    r["member_days_per_s"] = r["sim_days_per_s"]
                    r["ensemble_sim_days_per_s"] = r["sim_days_per_s"] / 512
                res["members"] = 512
            out["configs"][name] = res
            log(f"{name}: 1 thread {r1['ms_per_step']:.1f} ms/step, {cores} threads {rn['ms_per_step']:.1f} ms/step")
        elif name == "mixed":
            res = {"members_per_level": 16, "levels": {}}
            cyc = {1: 0.0, cores: 0.0}
            for L in (4, 5, 6, 7):
                dt = 1200.0 / 2 ** (L - 4)
                n = int(1200.0 / dt)
                m = mesh.generate_icos(L, 20)
                gd, u, ghs = cases.jet_bumps(m, seed=0)
                lv = {}
                for th in (1, cores):
                    r = _rate(m, gd, u, ghs, None, dt, n, th, repeats)
                    lv["single_thread" if th == 1 else "all_cores"] = r
                    cyc[th] += 16 * r["s_median"]  # 16 members, n steps each per cycle
                res["levels"][L] = lv
            for th, key in ((1, "single_thread"), (cores, "all_cores")):
                res[key] = {"s_per_cycle": cyc[th], "member_days_per_s": 64 * 1200.0 / DAY / cyc[th]}
            out["configs"][name] = res
            log(f"mixed: 1 thread {cyc[1]:.2f} s/cycle, {cores} threads {cyc[cores]:.2f} s/cycle")
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--repeats", type=int, default=3)
    ap.add_argument("--configs", default="level5,level9,ens512,mixed")
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    res = run(a.repeats, tuple(a.configs.split(",")), log=lambda s: print(s, file=sys.stderr, flush=True))
    txt = json.dumps(res)
    if a.out:
        with open(a.out, "w") as f:
            f.write(txt)
    print(txt)


if __name__ == "__main__":
    main()
