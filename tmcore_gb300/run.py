"""Run the shallow-water model on a generated icosahedral mesh and print one
JSON line: device ms per step (CUDA graph steps, CUDA events on the library
stream), ms per launch of each pass of the fused CRK4 step, and the
invariants before and after.

    python -m tmcore_gb300.run --level 8 --precision 64 --steps 3
    python -m tmcore_gb300.run --level 9 --precision 32 --tracers 4 --dt 45 --steps 10
    python -m tmcore_gb300.run --level 6 --case jet_zonal_flow --pv-scheme 3 --dt 240   # the shipped namelist
    python -m tmcore_gb300.run --level 6 --members 512 --member-layout 1 --steps 10      # an FP32 ensemble

An ensemble's members start from seeds seed, seed + 1, ... of the chosen case.
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import abi, cases
from .gpu import TMCoreGPU
from .mesh import icos_mesh


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--level", type=int, default=6)
    ap.add_argument("--precision", type=int, choices=(32, 64), default=32)
    ap.add_argument("--dt", type=float, default=0.0, help="0: 1200 / 2^(level-4) s")
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--tracers", type=int, default=0)
    ap.add_argument("--pv-scheme", type=int, default=1)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--case", default="jet_bumps", choices=cases.SWM_CASES)
    ap.add_argument("--autotune", action="store_true")
    ap.add_argument("--members", type=int, default=1, help="FP32 ensemble members (seeds seed, seed + 1, ...)")
    ap.add_argument("--member-layout", type=int, choices=(0, 1), default=1)
    a = ap.parse_args()
    m = icos_mesh(a.level)
    dt = a.dt if a.dt > 0 else 1200.0 / 2 ** (a.level - 4)
    prec = abi.TMC_FP32 if a.precision == 32 else abi.TMC_FP64
    kw = dict(interp_pv_order=3) if a.pv_scheme == 3 else dict(apvm_weight=0.0)
    if a.members > 1:
        kw.update(members=a.members, member_layout=a.member_layout)
    g = TMCoreGPU(m, dt=dt, precision=prec, pv_scheme=a.pv_scheme, adv_order=2, n_tracers=a.tracers,
                  diag_every=1, **kw)
    for k in range(a.members):
        gd, u, ghs = cases.by_name(a.case, m, seed=a.seed + k)
        if a.members > 1:
            g.select_member(k)
        g.set_initial(gd, u, ghs)
        if a.tracers:
            g.set_tracers(cases.smooth_tracers(m, a.tracers, seed=a.seed + k) * gd[None, :])
    if a.members > 1:
        g.select_member(0)
    d0 = g.diag()
    sizes = g.autotune(2) if a.autotune else None
    g.step(a.warmup)
    g.synchronize()
    ms, _, _, launches = g.time_steps(a.steps, total=True, flux=False)
    passes = g.pass_times(2)
    d1 = g.diag()
    g.close()
    print(json.dumps({"level": a.level, "case": a.case, "nCells": m.nCells, "members": a.members,
                      "member_layout": a.member_layout if a.members > 1 else None, "precision": a.precision, "dt_s": dt,
                      "tracers": a.tracers, "steps": a.steps, "ms_per_step": ms / a.steps,
                      "sim_days_per_s": dt / 86400.0 / (ms / a.steps / 1e3),
                      "member_days_per_s": a.members * dt / 86400.0 / (ms / a.steps / 1e3), "passes_ms": passes,
                      "gpu_launches": launches, "block_sizes": sizes,
                      "mass_rel_change": float((d1[0] - d0[0]) / d0[0]), "finite": bool(np.all(np.isfinite(d1)))}))


if __name__ == "__main__":
    main()
