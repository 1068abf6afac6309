"""Spreading independent picture pairs over ranks (one process per GPU) and combining the
per-frame results into per-sequence averages.

Every (frame, view) pair of the metric path is independent: there is no exchange step on the
device. A rank measures the pairs `shard_units` gives it; the per-sequence average of a
metric (xMetricStat::calcAvgMetric, apps/QMIV/src/xAppQMIV.h:256-260: compensated sum over
frames / number of frames) is formed on the host from all ranks' per-frame values, in frame
order, so it is identical to the single-process result whatever the number of ranks.
"""


def shard_units(areas, rank, world):
    """Indices of the units (picture pairs, given by their luma areas) that `rank` of `world`
    measures: longest-first greedy assignment to the least loaded rank, ties to the lowest
    rank and the lowest index. Deterministic, disjoint and complete over the ranks."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d of world %d" % (rank, world))
    order = sorted(range(len(areas)), key=lambda i: (-areas[i], i))
    load = [0] * world
    mine = []
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        load[r] += areas[i]
        if r == rank:
            mine.append(i)
    return sorted(mine)


def kbns_sum(values):
    """Compensated (Kahan-Babuska-Neumaier) sum in the reference's order (xKBNS,
    libs/pmbb-core/src/xMathUtils.h:16-103)."""
    s, c = 0.0, 0.0
    for v in values:
        t = s + v
        if abs(s) >= abs(v):
            c += (s - t) + v
        else:
            c += (v - t) + s
        s = t
    return s + c


def sequence_means(local_frames, group=None):
    """Per-sequence means of per-frame metric values held by different ranks.

    local_frames: {frame_index: {metric_name: value}} measured on this rank. All ranks call
    this collectively (torch.distributed all_gather_object on `group`); with no process group
    initialised it works on the local frames alone. Returns {metric_name: mean} over every
    frame of every rank, summed in frame order."""
    gathered = [local_frames]
    try:
        import torch.distributed as dist
        if dist.is_available() and dist.is_initialized():
            gathered = [None] * dist.get_world_size(group)
            dist.all_gather_object(gathered, local_frames, group=group)
    except ImportError:
        pass
    frames = {}
    for part in gathered:
        for f, vals in part.items():
            if f in frames:
                raise ValueError("frame %r measured on more than one rank" % (f,))
            frames[f] = vals
    if not frames:
        return {}
    names = sorted(set().union(*(v.keys() for v in frames.values())))
    order = sorted(frames)
    out = {}
    for n in names:
        vals = [frames[f][n] for f in order if n in frames[f]]
        out[n] = kbns_sum(vals) / len(vals)
    return out
