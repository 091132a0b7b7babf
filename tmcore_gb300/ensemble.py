"""Run an FP32 ensemble of one generated mesh, optionally with the learned
closure, and print the step time (CUDA events on the library stream).

    python -m tmcore_gb300.ensemble --members 512 --level 6 --steps 20
    python -m tmcore_gb300.ensemble --members 32 --closure --steps 3
    python -m tmcore_gb300.ensemble --members 512 --layout 1 --pv-scheme 3   # upwind pv, order 3
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import abi, cases, tune
from .gpu import ClosureMLP, TMCoreGPU
from .mesh import icos_mesh


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--members", type=int, default=64)
    ap.add_argument("--level", type=int, default=6)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--closure", action="store_true", help="a closure network of the trained shape on every stage")
    ap.add_argument("--autotune", action="store_true")
    ap.add_argument("--distinct-seeds", action="store_true", help="seed m for member m (else one seed for all)")
    ap.add_argument("--layout", type=int, default=0, help="member_layout: 0 member-outermost, 1 member-innermost")
    ap.add_argument("--pv-scheme", type=int, default=1, choices=(1, 3),
                    help="1 centred pv (APVM weight 0), 3 upwind pv (interp_pv_order 3)")
    ap.add_argument("--tune-ordering", action="store_true",
                    help="time element orders x member layouts first (tune.autotune_ordering) and use the fastest")
    a = ap.parse_args()
    m = icos_mesh(a.level)
    dt = 1200.0 / 2 ** (a.level - 4)
    ic = None if a.distinct_seeds else cases.jet_bumps(m, seed=0)
    ics = [cases.jet_bumps(m, seed=k) if a.distinct_seeds else ic for k in range(a.members)]
    pv = dict(pv_scheme=1, apvm_weight=0.0) if a.pv_scheme == 1 else dict(pv_scheme=3, interp_pv_order=3)
    params = dict(members=a.members, dt=dt, precision=abi.TMC_FP32, adv_order=2, diag_every=1,
                  member_layout=a.layout, **pv)
    orderings = None
    if a.tune_ordering:
        params, orderings = tune.autotune_ordering(m, ics, **params)
    ens = TMCoreGPU(m, **params)
    for k, (gd, u, ghs) in enumerate(ics):
        ens.select_member(k)
        ens.set_initial(gd, u, ghs)
    net = None
    if a.closure:
        net = ClosureMLP(seed=1)
        net.set_scaling(np.zeros(24), np.ones(24), 1e-12)
        ens.set_closure(net)
    sizes = ens.autotune(2) if (a.autotune or a.tune_ordering) else None
    ens.step(a.warmup)
    ens.synchronize()
    ms, _, _, launches = ens.time_steps(a.steps, total=True, flux=False)
    print(json.dumps({"members": a.members, "level": a.level, "layout": params["member_layout"],
                      "pv_scheme": a.pv_scheme,
                      "renumber": params.get("renumber", 1), "orderings": orderings, "closure": a.closure,
                      "ms_per_step": ms / a.steps,
                      "member_days_per_s": a.members * a.steps * dt / 86400.0 / (ms / 1e3),
                      "gpu_launches": launches, "block_sizes": sizes,
                      "closure_timed_out": ens.closure_status() if a.closure else None}))
    ens.close()
    if net is not None:
        net.close()


if __name__ == "__main__":
    main()
