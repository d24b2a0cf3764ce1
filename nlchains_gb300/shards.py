"""Copies sharded over processes, one GPU each: the reference's MPI decomposition without MPI.

The reference splits the ensemble's copies evenly over its MPI ranks (main.cpp:83-85 rejects a
copy count that is not a multiple of the rank count).  Each rank integrates its own chains; at
every sample the ranks sum their linear energies with an all_reduce (results_entropy.cpp:13), each
rank having normalised by the global copy count, and the entropies come from the summed vector.

Here each process runs its shard through a plan or job of `count` copies, whose linear energies
are normalised by that local count.  `combine_linenergies` rescales them to the global count and
sums them over a torch.distributed process group (gloo on host tensors: the exchange is N doubles
per sample, nothing on the data path); `sample` adds the entropies of the combined vector.
"""
import numpy as np

from . import entropies


def shard_range(copies, rank, world):
    """(first copy, copy count) of `rank` among `world` equal shards."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    if copies % world:
        raise ValueError("copies must be a multiple of the number of devices")   # main.cpp:84
    count = copies // world
    return rank * count, count


def combine_linenergies(lin_local, local_copies, total_copies, group=None):
    """Ensemble-average linear energies over every process of `group` (the default group when None,
    no exchange without torch.distributed): each process passes the energies of its own shard,
    normalised by its `local_copies`."""
    lin = np.asarray(lin_local, dtype=np.float64) * (float(local_copies) / float(total_copies))
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return lin
    t = torch.from_numpy(np.ascontiguousarray(lin))
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.numpy()


def sample(lin_local, local_copies, total_copies, a0is0, entropy_mask=None, group=None):
    """(combined linear energies, WT entropy, information entropy) of one sample."""
    lin = combine_linenergies(lin_local, local_copies, total_copies, group)
    wt, inf = entropies(lin, a0is0, entropy_mask)
    return lin, wt, inf
