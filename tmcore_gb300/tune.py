"""Ordering autotuner: picks how the device state is ordered for one
configuration, by timing it.

Two orderings are tuned, each fixed when a handle is created:

* element order (`renumber`): 1 Hilbert curve, 2 Morton curve of the unit-sphere
  positions, 0 the caller's (mesh file) order;
* for ensembles, the member layout (`member_layout`): 0 member-outermost
  (member = blockIdx.y), 1 member-innermost (arrays [element][member]), where
  its kernels apply; and for member_layout 1 the lanes of a warp per element
  (`member_lanes`: 8, 16 or 32, and with it one or two members per lane).

Each candidate is created with the same parameters and initial states. Its
block sizes are tuned by tmc_autotune, then `steps` CUDA-graph steps are timed
with CUDA events. Block sizes are tuned per candidate because the best block
size depends on the ordering.

    from tmcore_gb300 import tune
    best, timings = tune.autotune_ordering(mesh, ics, precision=1, members=512, dt=300.0)
"""
from __future__ import annotations

from .gpu import TMCError, TMCoreGPU

ORDERS = (1, 2, 0)
LANES = (0, 8, 16, 32)


def lane_layout(members: int, lanes: int):
    """(members per lane, lanes per element) of member_layout 1 for
    `member_lanes` = lanes (0: automatic), or None when lanes does not fit
    (the library's rule, tmc_ensemble.cuh lanes_for)."""
    if lanes == 0:
        return (2 if members % 64 == 0 else 1, 32 if members % 32 == 0 else 16)
    if lanes not in (8, 16, 32) or members % lanes:
        return None
    return (2 if members % (2 * lanes) == 0 else 1, lanes)


def lane_candidates(members: int, lanes=LANES):
    """The member_lanes values worth timing: one per distinct lane layout."""
    out, seen = [], set()
    for k in lanes:
        lay = lane_layout(members, k)
        if lay is not None and lay not in seen:
            seen.add(lay)
            out.append(k)
    return out


def autotune_ordering(mesh, ics, steps: int = 3, orders=ORDERS, layouts=None, lanes=LANES, **params):
    """Time every candidate ordering; return (best, timings).

    ics: one (gd, u, ghs) per member; params: TMCoreGPU keyword arguments
    (members defaults to len(ics)).  best: params with the `renumber`,
    `member_layout` and `member_lanes` of the fastest candidate; timings: one
    dict per candidate (renumber, member_layout, member_lanes, ms_per_step,
    block_sizes), or the error when the candidate cannot be built (an option
    its kernels lack)."""
    members = int(params.pop("members", len(ics)))
    if layouts is None:
        layouts = (1, 0) if members > 1 else (0,)
    cands = [(layout, order, ln) for layout in layouts for order in orders
             for ln in (lane_candidates(members, lanes) if layout == 1 else [0])]
    timings, best = [], None
    for layout, order, ln in cands:
        kw = dict(params, members=members, renumber=order, member_layout=layout, member_lanes=ln)
        try:
            g = TMCoreGPU(mesh, **kw)
        except TMCError as e:
            timings.append({"renumber": order, "member_layout": layout, "member_lanes": ln, "error": str(e)})
            continue
        try:
            for m, (gd, u, ghs) in enumerate(ics):
                g.select_member(m)
                g.set_initial(gd, u, ghs)
            sizes = g.autotune(2)
            g.step(1)
            g.synchronize()
            ms, _, _, _ = g.time_steps(steps, total=True, flux=False)
        finally:
            g.close()
        t = {"renumber": order, "member_layout": layout, "member_lanes": ln, "ms_per_step": ms / steps,
             "block_sizes": sizes}
        timings.append(t)
        if best is None or t["ms_per_step"] < best["ms_per_step"]:
            best = t
    if best is None:
        raise TMCError(-4, "no ordering candidate could be built for these parameters")
    out = dict(params, members=members, renumber=best["renumber"], member_layout=best["member_layout"],
               member_lanes=best["member_lanes"])
    return out, timings
