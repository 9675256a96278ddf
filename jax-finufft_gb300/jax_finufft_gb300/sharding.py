"""Data-parallel NUFFTs over the nonuniform points, one rank per GPU.

The reference distributes its transforms with ``jax.shard_map`` (README.md
"Sharding", 339-437): the nonuniform points (and their strengths) are
sharded, the uniform grid is replicated, and each transform type combines the
ranks' local results with at most one collective:

=================  ======================  =====================  ===========================
transform          sharded                 replicated             combine
=================  ======================  =====================  ===========================
type 1             points + strengths      --                     sum of the N-mode outputs
type 2             points                  grid                   none
type 3 (sources)   sources + strengths     targets                sum of the outputs
type 3 (targets)   targets                 sources + strengths    none
=================  ======================  =====================  ===========================

Sharding both sides of a type 3 is not supported (tests/sharding_test.py:
292-334 keeps it as a strict xfail).  This module is that recipe for
``torch.distributed`` process groups:

* a summed output goes through :func:`reduce_sum` -- an all-reduce forward
  whose backward passes the cotangent through unchanged, since the loss
  downstream of a replicated output is evaluated identically on every rank;
* a replicated input goes through :func:`replicated` -- identity forward,
  all-reduce of the cotangent backward, the psum that the reference gets from
  a ``pvary`` on a replicated input (src/jax_finufft/ops.py:34-47,
  reconcile_vma), so the gradient of the replicated grid (type 2) or of
  replicated sources (type 3, target-sharded) is the sum over every rank's
  points.

The per-rank transform defaults to this package's nufft1/2/3 (the GPU path);
``transform`` replaces it (any callable with the same signature), which the
CPU tests use.  Every rank must call these functions in the same order (each
collective is a matching call on all ranks).
"""
import torch
import torch.distributed as dist

__all__ = ["reduce_sum", "replicated", "nufft1", "nufft2", "nufft3"]


class _ReduceSum(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, group):
        y = x.clone()
        dist.all_reduce(y, op=dist.ReduceOp.SUM, group=group)
        return y

    @staticmethod
    def backward(ctx, g):
        return g, None


class _Replicated(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, group):
        ctx.group = group
        return x.view_as(x)

    @staticmethod
    def backward(ctx, g):
        g = g.clone()
        dist.all_reduce(g, op=dist.ReduceOp.SUM, group=ctx.group)
        return g, None


def reduce_sum(x, group=None):
    """Sum of x over the ranks of group (every rank gets the sum)."""
    return _ReduceSum.apply(x, group)


def replicated(x, group=None):
    """Mark x as replicated on every rank: its gradient is summed over ranks."""
    if not (torch.is_tensor(x) and x.requires_grad):
        return x
    return _Replicated.apply(x, group)


def _default(name):
    from . import ops

    return getattr(ops, name)


def nufft1(output_shape, source, *points, group=None, transform=None, **kwargs):
    """Type 1 with the points and strengths sharded: each rank spreads its
    own points, the N-mode outputs are summed (README.md:376)."""
    fn = transform or _default("nufft1")
    return reduce_sum(fn(output_shape, source, *points, **kwargs), group)


def nufft2(source, *points, group=None, transform=None, **kwargs):
    """Type 2 with the grid replicated and the points sharded: each rank
    evaluates the grid at its own points, no collective (README.md:377)."""
    fn = transform or _default("nufft2")
    return fn(replicated(source, group), *points, **kwargs)


def nufft3(source, *points, shard="sources", group=None, transform=None, **kwargs):
    """Type 3 with one side sharded (README.md:378-379).

    shard="sources": strengths and source points sharded, targets
    replicated; the outputs are summed.  shard="targets": targets sharded,
    strengths and sources replicated; no forward collective.  points are
    the d source arrays followed by the d target arrays, as in nufft3."""
    fn = transform or _default("nufft3")
    if len(points) % 2:
        raise ValueError("nufft3 takes d source and d target coordinate arrays")
    d = len(points) // 2
    src, tgt = list(points[:d]), list(points[d:])
    if shard == "sources":
        tgt = [replicated(t, group) for t in tgt]
        return reduce_sum(fn(source, *src, *tgt, **kwargs), group)
    if shard == "targets":
        src = [replicated(s, group) for s in src]
        return fn(replicated(source, group), *src, *tgt, **kwargs)
    if shard == "both":
        raise NotImplementedError(
            "sharding both the sources and the targets of a type-3 transform is not "
            "supported: every target depends on every source")
    raise ValueError("shard must be 'sources' or 'targets'")
