"""Sharding of an ensemble of independent tanks over ranks (one GPU each).

The tanks of an ensemble share nothing, so the ensemble is split into
contiguous blocks of tanks, one block per rank, balanced by an estimate of
each tank's work.  Each rank advances its own block with
hosnwt_advance_many; no data crosses ranks while the tanks run.  At the end
the per-tank summaries (final time, step counts, probe values) are gathered
on rank 0 in tank order, the only collective of the ensemble.

Work estimate of one tank (transform FMAs scale as n1 log n1 per transform,
with about M^2 transforms per right-hand side), times its number of RK
steps over the simulated time:

    cost = n1 * log2(n1) * M^2 * steps,
    steps = T_sim / (0.95 * dt_stab),

with dt_stab the reference's RK4 stability limit (HOS-NWT.f90:131-186):
the smaller of sqrt(8/pi^2) xlen/(n1-1) (x modes) and
sqrt(8/pi^2) 2 l_add/(l_add (n3-1)) (wavemaker z modes, l_add = 2) for a
2-D tank with a wavemaker, in units of the depth and sqrt(h/g).
"""
from __future__ import annotations

import math

G = 9.81


def rk4_stability_dt(n1, n3, xlen, h, has_wavemaker=True):
    """Nondimensional RK4 stability step of HOS-NWT.f90:131-186 for a 2-D
    tank (n2 = 1), lengths in metres."""
    c = math.sqrt(8.0 / math.pi ** 2)
    dt_x = c * (xlen / h) / (n1 - 1)
    if not has_wavemaker:
        return dt_x
    l_add = 2
    dt_z = c * (2.0 * l_add) / (l_add * (n3 - 1))
    return min(dt_x, dt_z)


def tank_steps(spec, sim_seconds):
    """Estimated RK steps of one tank over `sim_seconds` of simulated time."""
    inp = spec["inp"]
    h = float(inp.get("h", 5.0))
    tscale = math.sqrt(h / G)
    dt = 0.95 * rk4_stability_dt(int(spec["n1"]), int(spec["n3"]), float(inp.get("xlen", 50.0)), h,
                                 int(inp.get("igeom", 2)) != 3)
    dt = min(dt, 1.0 / float(inp.get("f_out", 10.0)) / tscale)
    return sim_seconds / (dt * tscale)


def tank_cost(spec, sim_seconds):
    """Work estimate of one tank: n1 log2(n1) M^2 x steps."""
    n1, M = int(spec["n1"]), int(spec["mHOS"])
    return n1 * math.log2(n1) * M * M * tank_steps(spec, sim_seconds)


def partition(costs, world):
    """Contiguous blocks [start, stop) of the tanks, one per rank, that
    balance the summed cost: block r ends where the running cost first
    reaches (r + 1) / world of the total (nearer of the two neighbouring
    cuts).  Every tank lands in exactly one block; a block may be empty when
    there are fewer tanks than ranks."""
    n = len(costs)
    if world < 1:
        raise ValueError("world must be >= 1")
    if any(c < 0 for c in costs):
        raise ValueError("costs must be non-negative")
    total = float(sum(costs))
    prefix = [0.0]
    for c in costs:
        prefix.append(prefix[-1] + float(c))
    cuts = [0]
    for r in range(1, world):
        target = total * r / world
        # first index i with prefix[i] >= target, at or after the previous cut
        i = cuts[-1]
        while i < n and prefix[i] < target:
            i += 1
        if i > cuts[-1] and abs(prefix[i - 1] - target) < abs(prefix[i] - target):
            i -= 1
        # leave at least one tank for each remaining rank when possible
        i = min(i, n - (world - r)) if n >= world else i
        cuts.append(max(i, cuts[-1]))
    cuts.append(n)
    return [(cuts[r], cuts[r + 1]) for r in range(world)]


def shard(specs, rank, world, sim_seconds):
    """The block [start, stop) of tanks that `rank` of `world` runs."""
    return partition([tank_cost(s, sim_seconds) for s in specs], world)[rank]


def gather_summaries(local, start, n_total, group=None):
    """Gather per-tank summaries (one dict per tank of this rank's block,
    starting at tank index `start`) on rank 0, in tank order.  Returns the
    full list on rank 0 and None elsewhere; with no process group, returns
    the local list."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return list(local)
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    parts = [None] * world if rank == 0 else None
    dist.gather_object((start, list(local)), parts, dst=0, group=group)
    if rank != 0:
        return None
    out = [None] * n_total
    for st, items in parts:
        for i, s in enumerate(items):
            if out[st + i] is not None:
                raise RuntimeError(f"tank {st + i} reported by two ranks")
            out[st + i] = s
    missing = [i for i, s in enumerate(out) if s is None]
    if missing:
        raise RuntimeError(f"tanks {missing} were not reported by any rank")
    return out
