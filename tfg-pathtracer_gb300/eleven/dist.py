"""Several processes (one per GPU) rendering one image.

Samples are independent and their random numbers depend only on (pixel,
sample index, seed), so a render of `spp` samples splits into disjoint
sample ranges, one per rank (`er_render_opts.sample_begin`), and the films
combine as sample-count-weighted means.  No data moves during a render; the
one exchange is the final film reduction.

The reference renders one process per scene and has no multi-GPU path
(kernel.cu:665-686 loops over samples on one device), so this is the
replica form: `shard_samples` picks a rank's range, `reduce_film` merges the
ranks' films with two all-reduce sums (torch.distributed, any backend:
gloo on CPU tensors, NCCL on CUDA tensors).
"""
import numpy as np


def shard_samples(spp, rank, world, sample_begin=0):
    """(first sample, count) of `rank`'s share of [sample_begin,
    sample_begin + spp): contiguous ranges, the first spp % world ranks one
    sample longer."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank out of range")
    if spp < 0:
        raise ValueError("negative sample count")
    q, r = divmod(spp, world)
    count = q + (1 if rank < r else 0)
    first = sample_begin + rank * q + min(rank, r)
    return first, count


def merge_films(beauties, samples):
    """Sample-count-weighted mean of films ((H*W, 4) float32 RGBA beauty,
    (H*W,) per-pixel sample counts), in float64; alpha stays 1."""
    num = np.zeros(beauties[0].shape[:1] + (3,), np.float64)
    cnt = np.zeros(beauties[0].shape[0], np.float64)
    for b, s in zip(beauties, samples):
        s = np.asarray(s, np.float64)
        num += np.asarray(b, np.float64)[:, :3] * s[:, None]
        cnt += s
    out = np.ones(beauties[0].shape, np.float32)
    with np.errstate(invalid="ignore", divide="ignore"):
        out[:, :3] = np.where(cnt[:, None] > 0, num / np.maximum(cnt, 1)[:, None], 0.0)
    return out, cnt.astype(np.uint32)


def reduce_film(beauty, samples, group=None):
    """All-reduce of one rank's film with the other ranks' (every rank gets
    the merged film): sums of beauty * samples and of samples in float64.
    beauty (H*W, 4) and samples (H*W,) as numpy arrays or torch tensors; a
    CUDA tensor stays on its device (NCCL), anything else reduces on the CPU
    (gloo).  Returns (beauty float32 with alpha 1, samples) like the inputs'
    kind."""
    import torch
    import torch.distributed as dist
    is_t = torch.is_tensor(beauty)
    b = beauty if is_t else torch.from_numpy(np.ascontiguousarray(beauty))
    s = samples if torch.is_tensor(samples) else torch.from_numpy(np.ascontiguousarray(samples).astype(np.int64))
    s64 = s.to(torch.float64)
    num = b[:, :3].to(torch.float64) * s64[:, None]
    dist.all_reduce(num, group=group)
    dist.all_reduce(s64, group=group)
    out = torch.ones_like(b, dtype=torch.float32)
    out[:, :3] = torch.where(s64[:, None] > 0, num / s64.clamp(min=1)[:, None], torch.zeros_like(num)).float()
    cnt = s64.round().to(torch.int64)
    if is_t:
        return out, cnt
    return out.numpy(), cnt.numpy().astype(np.uint32)


def reduce_sums(sums, samples, group=None):
    """All-reduce of one rank's exact film (the FP64 per-pixel sums and
    sample counts of an ER_RENDER_ACCUM_FP64 render, er_film_read_sums):
    every rank gets the summed sums and counts, and the merged beauty (the
    FP64 means rounded once to float32, alpha 1).  Unlike reduce_film no
    rank's mean is rounded before the merge, so the result equals one
    process rendering every sample in FP64 up to the order of the additions."""
    import torch
    import torch.distributed as dist
    is_t = torch.is_tensor(sums)
    sm = sums.to(torch.float64) if is_t else torch.from_numpy(np.ascontiguousarray(sums, np.float64))
    s64 = (samples if torch.is_tensor(samples) else torch.from_numpy(np.ascontiguousarray(samples).astype(np.int64)))
    s64 = s64.to(torch.float64)
    dist.all_reduce(sm, group=group)
    dist.all_reduce(s64, group=group)
    beauty = torch.ones((sm.shape[0], 4), dtype=torch.float32, device=sm.device)
    beauty[:, :3] = torch.where(s64[:, None] > 0, sm / s64.clamp(min=1)[:, None], torch.zeros_like(sm)).float()
    cnt = s64.round().to(torch.int64)
    if is_t:
        return sm, cnt, beauty
    return sm.numpy(), cnt.numpy().astype(np.uint32), beauty.numpy()
