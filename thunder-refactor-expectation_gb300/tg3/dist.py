"""The exchange of the insertion over ranks, when particles are sharded over
GPUs (one process per GPU).

The E-step needs no exchange: every rank scores its own particles against
its own copy of the reference volumes (the reference replicates them per
GPU, src/Optimiser.cpp:2252-2345).  The insertion ends with one sum: every
rank inserts its own particles into its accumulators, then F, T, O3D and
the counter are summed over the ranks of a half map (the reference:
ncclAllReduce of F and T over the hemisphere, gpu/src/cuthunder.cu:4956-5000,
and Reconstructor::allReduceF / allReduceT / allReduceO,
src/Reconstructor.cpp:2348-2500).  The sums are plain element-wise
reductions of the accumulator arrays, done in place with torch.distributed
(NCCL between GPUs, gloo on CPU); tg3.Context.insert_read hands a rank's
accumulators out and Context.insert_load takes the sums back in for the
reconstruction.
"""
from __future__ import annotations


def allreduce_insertion(F, T, O3D=None, counter=None, group=None):
    """Sum the insertion accumulators of every rank of `group` in place:
    F (complex half volume, or its float pairs), T (real), and when given
    O3D [3] (float64) and counter (integer).  Every rank must call it with
    arrays of the same shapes and dtypes (torch tensors on the process
    group's device kind)."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        raise RuntimeError("allreduce_insertion needs an initialised process group")
    Fr = torch.view_as_real(F) if F.is_complex() else F
    for x in (Fr, T) + tuple(v for v in (O3D, counter) if v is not None):
        if not x.is_contiguous():
            raise ValueError("accumulators must be contiguous")
        dist.all_reduce(x, op=dist.ReduceOp.SUM, group=group)
    return F, T, O3D, counter
