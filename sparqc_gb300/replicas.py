"""Independent replicas on several GPUs: placement of circuits and reduction of the timings.

Circuits are independent, so several GPUs share a workload with no exchange on the data path
(the reference's own multi-GPU layouts are unbuilt stubs, emulator/device/device_table_FCS.cuh).
Each rank runs its shard on its own GPU; only the step time (max over ranks) and the work done
(sum over ranks) cross ranks, once per measurement, through torch.distributed.
"""

from .gates import H, RX, RY, U, X, Y

BRANCH = (H, RX, RY, U)
SWAP = (X, Y)


def varying_bits(nq, gates):
    """Bits that can ever differ between keys of a circuit started from |0...0>: the host
    planner's known-bit tracking (sparqc_gb300/csrc/sqc_plan.cpp, plan_gate) restated. A gate
    with a control known to be 0 does nothing; an X or Y whose controls are all known to be 1
    relabels a known bit; any other branching or swap gate makes its target vary."""
    known = (1 << nq) - 1   # bits known to be equal across keys
    val = 0                  # their value
    for g in gates:
        kind, target, controls = int(g["kind"]), int(g["target"]), int(g["controls"])
        kc = controls & known
        if (val & kc) != kc:
            continue
        unknown_ctrl = controls & ~known
        bit = 1 << target
        if kind in SWAP and not unknown_ctrl:
            if known & bit:
                val ^= bit
            continue
        if kind in BRANCH or kind in SWAP:
            known &= ~bit
    return [q for q in range(nq) if not (known >> q) & 1]


def circuit_cost(nq, gates):
    """Estimated (table bytes, work) of one circuit from |0...0>: keys <= 2^(varying bits),
    groups <= 2^(varying bits >= 4), work ~ keys x gates."""
    v = varying_bits(nq, gates)
    groups = 2 ** len([q for q in v if q >= 4])
    keys = 2 ** len(v)
    return groups * 16 * 24 * 2, keys * max(1, len(gates))


def shard(circuits, rank, world):
    """Indices of the circuits rank `rank` of `world` runs: longest-processing-time-first over
    the estimated work, deterministic, so every rank computes the same placement without
    communicating."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("bad rank/world")
    costs = [circuit_cost(nq, g)[1] for nq, g in circuits]
    order = sorted(range(len(circuits)), key=lambda i: (-costs[i], i))
    load = [0] * world
    owner = [0] * len(circuits)
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        owner[i] = r
        load[r] += costs[i]
    return [i for i in range(len(circuits)) if owner[i] == rank]


def reduce_step(seconds, work, group=None):
    """(max seconds over ranks, total work over ranks) of one measurement."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return seconds, work
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor([seconds], dtype=torch.float64, device=dev)
    w = torch.tensor([float(work)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    dist.all_reduce(w, op=dist.ReduceOp.SUM, group=group)
    return float(t.item()), float(w.item())


def imbalance(circuits, world):
    """max/mean estimated work over ranks of the placement (1.0 = perfect)."""
    per = [sum(circuit_cost(*circuits[i])[1] for i in shard(circuits, r, world)) for r in range(world)]
    mean = sum(per) / world
    return max(per) / mean if mean > 0 else 1.0
