"""One search spread over several GPUs, one process per GPU.

The reference's single call uses every visible GPU: one OpenMP thread per
device, every device holding the whole data, templates claimed from a shared
counter (matched_filter.cu:186-224, 261-280).  Templates are independent, so
here each GPU is driven by its own process (torchrun, one rank per GPU):
``template_block`` gives rank r of W a contiguous block of the templates,
``matched_filter_sharded`` runs the search on that block on the rank's GPU
and, when asked, gathers every rank's rows into the whole result.  Nothing
moves between ranks during the search; the gather is the only exchange.
"""
import numpy as np

from .fast_matched_filter import _infer_dims, matched_filter


def template_block(n_templates, world, rank):
    """[t0, t1) of rank ``rank`` out of ``world``: contiguous blocks whose
    sizes differ by at most one, the larger ones first.  Ranks beyond the
    template count get empty blocks."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d of world size %d" % (rank, world))
    base, extra = divmod(int(n_templates), world)
    t0 = rank * base + min(rank, extra)
    return t0, t0 + base + (1 if rank < extra else 0)


def _dist_rank_world(rank, world):
    if rank is not None and world is not None:
        return rank, world
    try:
        import torch.distributed as dist
        if dist.is_available() and dist.is_initialized():
            return dist.get_rank(), dist.get_world_size()
    except ImportError:
        pass
    return 0, 1


def _gather_rows(block, n_templates, world, rank):
    """Every rank's block of rows, in rank order, on every rank (all-gather
    padded to the largest block; CUDA tensors under NCCL, CPU under gloo)."""
    import torch
    import torch.distributed as dist
    rows = [template_block(n_templates, world, r) for r in range(world)]
    most = max(t1 - t0 for t0, t1 in rows)
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" \
        else torch.device("cpu")
    pad = torch.zeros((most,) + block.shape[1:], dtype=torch.float32, device=dev)
    pad[:block.shape[0]] = torch.from_numpy(np.ascontiguousarray(block)).to(dev)
    parts = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad)
    return np.concatenate([p[:t1 - t0].cpu().numpy() for p, (t0, t1) in zip(parts, rows)])


def matched_filter_sharded(templates, moveouts, weights, data, step, rank=None, world=None,
                           gather=True, search=None, **kwargs):
    """``matched_filter`` over this rank's block of templates.

    templates, moveouts, weights carry the template axis first (the
    reference's multi-template formats); data is the whole trace on every
    rank.  rank / world default to torch.distributed's (a single process
    when it is not initialised).  Returns the whole (T, n_corr[, S, C])
    result when ``gather`` (every rank gets it), else this rank's rows
    together with their template range: (rows, (t0, t1)).  ``search`` is the
    per-block search function (default: this package's GPU matched_filter;
    keyword arguments are passed on to it).
    """
    rank, world = _dist_rank_world(rank, world)
    dims = _infer_dims(np.asarray(templates), np.asarray(data))
    if dims is None or np.asarray(templates).ndim <= np.asarray(data).ndim:
        raise ValueError("templates need a leading template axis to be sharded")
    T = dims[0]
    t0, t1 = template_block(T, world, rank)
    search = search or matched_filter
    mo, w = np.asarray(moveouts), np.asarray(weights)
    if t1 > t0:
        rows = search(templates[t0:t1], mo[t0:t1], w[t0:t1], data, step, **kwargs)
    else:  # an idle rank: an empty block of the result's shape
        one = search(templates[:1], mo[:1], w[:1], data, step, **kwargs)
        rows = np.zeros((0,) + one.shape[1:], dtype=np.float32)
    rows = np.asarray(rows, dtype=np.float32)
    if not gather:
        return rows, (t0, t1)
    if world == 1:
        return rows
    return _gather_rows(rows, T, world, rank)
