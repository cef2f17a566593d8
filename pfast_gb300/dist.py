"""Sources sharded over processes (one GPU each).

The reference's only parallel strategy is source-level data parallelism over MPI
ranks: contiguous blocks of sources per rank (src/T_PFAST3D.cpp:221-236,
src/RT_PFAST2D.cpp:271-286), a full model replica per rank, and one exchange
step -- MPI_Allreduce(SUM) of the N-vector gradient and of the misfit
(src/T_PFAST3D.cpp:397-399).  This module keeps that partition and replaces the
reduction by a fixed-order sum over ranks (the result does not depend on the
collective's internal reduction order): rank r's partial gradient is the
source-ordered sum over its block, and the total is ((g_0 + g_1) + g_2) + ...

On a single GPU the library batches every source itself; this module is for
runs that shard a survey over several processes (torch.distributed, any backend).
"""
import numpy as np


def loc_srcid(nsrc, nranks):
    """Exclusive end of each rank's source block (src/T_PFAST3D.cpp:221-236): when nsrc is
    not divisible by nranks, the first nsrc % nranks ranks take one source more."""
    rmd = nsrc % nranks
    per = (nsrc - rmd) // nranks
    ends = []
    for r in range(nranks):
        if rmd:
            ends.append((r + 1) * (per + 1) if r < rmd else ends[r - 1] + per)
        else:
            ends.append((r + 1) * per)
    return ends


def source_block(nsrc, rank, nranks):
    """[begin, end) of rank's sources."""
    ends = loc_srcid(nsrc, nranks)
    return (ends[rank - 1] if rank > 0 else 0), ends[rank]


def ordered_sum(parts):
    """((p0 + p1) + p2) + ... elementwise, in float64."""
    acc = np.array(parts[0], dtype=np.float64, copy=True)
    for p in parts[1:]:
        acc = acc + np.asarray(p, dtype=np.float64)
    return acc


def reduce_gradient(grad_part, misfit_part, group=None):
    """Gather every rank's partial gradient and misfit and sum them in rank order on every
    rank (the reference's two MPI_Allreduce(SUM) calls with a fixed order).
    grad_part: float64 numpy array (host).  Returns (grad, misfit)."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    t = torch.from_numpy(np.ascontiguousarray(grad_part, dtype=np.float64).ravel())
    e = torch.tensor([float(misfit_part)], dtype=torch.float64)
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = t.to(dev)
    e = e.to(dev)
    gt = [torch.empty_like(t) for _ in range(world)]
    ge = [torch.empty_like(e) for _ in range(world)]
    dist.all_gather(gt, t, group=group)
    dist.all_gather(ge, e, group=group)
    grad = ordered_sum([g.cpu().numpy() for g in gt]).reshape(np.shape(grad_part))
    misfit = float(ordered_sum([x.cpu().numpy() for x in ge])[0])
    return grad, misfit


def sharded_eval3d(ctx, vp, dx, dy, dz, src, srnum, rec, nxyz, tobs, rank, nranks, group=None, **opts):
    """Misfit + gradient of a 3D survey sharded over ranks: this rank evaluates its block of
    sources on its GPU (pfast_eval3d), then the partial results are summed in rank order."""
    from .api import eval3d_host
    b, e = source_block(len(srnum), rank, nranks)
    ch = np.concatenate([[0], np.cumsum(srnum)])
    if e > b:
        g, m, _ = eval3d_host(ctx, vp, dx, dy, dz, src[b:e], srnum[b:e], rec[ch[b]:ch[e]], nxyz[ch[b]:ch[e]],
                              tobs[ch[b]:ch[e]], **opts)
    else:
        g, m = np.zeros_like(vp), 0.0
    return reduce_gradient(g, m, group)
