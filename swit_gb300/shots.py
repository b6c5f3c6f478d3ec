"""Shot sharding across ranks and the one exchange step of the path.

fd2dmpi splits shots into contiguous blocks per MPI rank (get_assigned,
fd2dmpi/mmi_mpi.f90:52-80) and sums the per-rank gradients and illuminations
with MPI_Allreduce (fd2dmpi/solver.f90:263-265).  Here one rank drives one GPU:
its block of shots is the batch of its engine, and the sum is one
torch.distributed all_reduce of the three (nx, nz) arrays.
"""


def assigned(ns, rank, world):
    """Half-open shot range [b, e) of `rank` among `world` ranks, as get_assigned."""
    if world == 1:
        return 0, ns
    nnn = ns
    ii1 = nnn // world
    if ii1 == 0:
        b = rank
        return (b, b + 1) if b < ns else (ns, ns)
    ii2 = nnn - ii1 * world
    if rank < world - ii2:
        b = rank * ii1
        e = (rank + 1) * ii1 - 1
    else:
        b = ii2 + rank * ii1 + rank - world
        e = ii2 + (rank + 1) * ii1 + rank - world
    return b, e + 1


def allreduce_sum(tensors, group=None):
    """Sums each tensor over all ranks in place (solver.f90:263-265)."""
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size(group) == 1:
        return tensors
    for t in tensors:
        dist.all_reduce(t, group=group)
    return tensors
