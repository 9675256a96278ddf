"""Broadcasting and flattening of NUFFT inputs, in torch.

Same rules as src/jax_finufft/shapes.py:11-170: point dimensions broadcast
over source dimensions are packed into the stacked-transform axis
(``n_transf``) so one setpts serves all of them; matched leading dimensions
become ``n_tot``.  The canonical buffers are
  types 1/3: source (n_tot, n_transf, M), points (n_tot, M)
  type 2:    source (n_tot, n_transf, N...), points (n_tot, M)
"""
from dataclasses import dataclass
from typing import Sequence

import numpy as np
import torch


@dataclass
class BroadcastIndex:
    broadcast_from: Sequence[int]
    broadcast_to: Sequence[int]
    expected_output_shape: Sequence[int]

    def unflatten(self, result):
        """Inverse of the flattening (shapes.py:17-24)."""
        out = torch.reshape(result, tuple(self.expected_output_shape))
        if len(self.broadcast_to):
            out = torch.movedim(out, tuple(self.broadcast_to), tuple(self.broadcast_from))
        return out


def _flat_vector_points(nufft_type, output_shape, source, points):
    """The common case of one point set, every point array 1-D of one length
    M: the general rules below reduce to reshapes (n_tot = 1; a source with
    one leading axis is that many stacked transforms).  None when the inputs
    are not of that form or disagree on the point count (the general path
    then checks and reports them).  Same results as the general path, in a
    few tensor operations instead of some twenty (per call that is most of
    a small transform's host time)."""
    if not all(isinstance(p, torch.Tensor) and p.ndim == 1 for p in points):
        return None
    m = points[0].shape[0]
    if any(p.shape[0] != m for p in points[1:]):
        return None
    if nufft_type == 3:
        num_dim = len(points) // 2
        src_pts, tgt_pts = points[:num_dim], points[num_dim:]
        n3 = tgt_pts[0].shape[0]
        if any(p.shape[0] != n3 for p in tgt_pts[1:]):
            return None
        if any(p.shape[0] != m for p in src_pts):
            return None
        extra = (m,)
        tail = (n3,)
    elif nufft_type == 2:
        num_dim = len(points)
        extra = tuple(source.shape[source.ndim - num_dim:]) if source.ndim >= num_dim else None
        tail = (m,)
        if extra is None:
            return None
    else:
        num_dim = len(points)
        extra = (m,)
        tail = tuple(output_shape) if output_shape is not None else None
        if tail is None:
            return None
    lead = source.ndim - len(extra)
    if lead == 0:
        n_transf, expected = 1, tail
    elif lead == 1:
        n_transf, expected = int(source.shape[0]), (int(source.shape[0]),) + tail
    else:
        return None
    if tuple(source.shape[lead:]) != extra:
        return None
    index = BroadcastIndex(broadcast_from=(), broadcast_to=(),
                           expected_output_shape=expected)
    flat = torch.reshape(source, (1, n_transf) + extra)
    return (index, flat) + tuple(p.reshape(1, p.shape[0]) for p in points)


def broadcast_and_flatten_inputs(nufft_type, output_shape, source, *points):
    """Port of shapes.py:27-126 (same dimension bookkeeping, torch ops)."""
    fast = _flat_vector_points(nufft_type, output_shape, source, points)
    if fast is not None:
        return fast
    if nufft_type == 3:
        num_dim = len(points) // 2
        points3 = points[num_dim:]
        points = points[:num_dim]
    else:
        num_dim = len(points)
    assert num_dim

    points = torch.broadcast_tensors(*points)
    *input_shape, num_points = points[0].shape
    input_shape = tuple(input_shape)

    if nufft_type == 3:
        points3 = torch.broadcast_tensors(*points3)
        *input_shape3, num_points3 = points3[0].shape
        input_shape = tuple(torch.broadcast_shapes(input_shape, tuple(input_shape3)))
        points = [p.expand(input_shape + (num_points,)) for p in points]
        points3 = [p.expand(input_shape + (num_points3,)) for p in points3]
    else:
        points3 = []

    # unpadded points
    if (nufft_type == 2 and source.ndim == len(input_shape) + num_dim + 1) or (
        nufft_type in (1, 3) and source.ndim == len(input_shape) + 2
    ):
        input_shape = tuple(input_shape) + (1,)
        points = tuple(p[..., None, :] for p in points)

    target_shape = tuple(torch.broadcast_shapes(tuple(source.shape[: len(input_shape)]),
                                                tuple(input_shape)))

    broadcast_from = tuple(
        n for n, (input_dim, target_dim) in enumerate(zip(input_shape, target_shape))
        if input_dim != target_dim
    )
    broadcast_to = tuple(
        len(target_shape) - len(broadcast_from) + n for n in range(len(broadcast_from))
    )
    assert all(input_shape[n] == 1 for n in broadcast_from)

    source = source.expand(target_shape + tuple(source.shape[len(target_shape):]))

    if len(broadcast_to):
        source = torch.movedim(source, broadcast_from, broadcast_to)
        points = tuple(torch.movedim(p, broadcast_from, broadcast_to) for p in points)
        points3 = tuple(torch.movedim(p, broadcast_from, broadcast_to) for p in points3)

    num_in = len(target_shape)
    num_axes = num_in - len(broadcast_from)
    size_in = int(np.prod(source.shape[:num_axes], dtype=np.int64))
    size_bcast = int(np.prod(source.shape[num_axes:num_in], dtype=np.int64))

    if nufft_type == 3:
        assert source.ndim == len(target_shape) + 1
        assert source.shape[-1] == num_points
        expected_output_shape = tuple(source.shape[:num_in]) + (num_points3,)
        source_extra_shape = (num_points,)
    elif nufft_type == 2:
        assert source.ndim == num_in + num_dim
        expected_output_shape = tuple(source.shape[:num_in]) + (num_points,)
        source_extra_shape = tuple(source.shape[num_in:])
    else:
        assert source.ndim == len(target_shape) + 1
        assert source.shape[-1] == num_points
        assert output_shape is not None
        expected_output_shape = tuple(source.shape[:num_in]) + tuple(output_shape)
        source_extra_shape = (num_points,)

    source = torch.reshape(source, (size_in, size_bcast) + tuple(source_extra_shape))
    points = tuple(torch.reshape(p, (size_in, num_points)) for p in points)
    points3 = tuple(torch.reshape(p, (size_in, num_points3)) for p in points3)

    return (
        BroadcastIndex(
            broadcast_from=broadcast_from,
            broadcast_to=broadcast_to,
            expected_output_shape=expected_output_shape,
        ),
        source,
        *points,
        *points3,
    )


def check_canonical(source, points, nufft_type):
    """Dtype and shape checks of shapes.abstract_eval (shapes.py:129-170)."""
    ndim = len(points) // 2 if nufft_type == 3 else len(points)
    if not 1 <= ndim <= 3:
        raise ValueError("Only 1-, 2-, and 3-dimensions are supported")
    single = source.dtype == torch.complex64 and all(p.dtype == torch.float32 for p in points)
    double = source.dtype == torch.complex128 and all(p.dtype == torch.float64 for p in points)
    if not (single or double):
        raise TypeError("inputs must be complex64 with float32 points, or complex128 with "
                        "float64 points; got %s and %s"
                        % (source.dtype, [str(p.dtype) for p in points]))
    if not all(p.ndim == 2 for p in points):
        raise ValueError("canonical points must be 2-D (n_tot, M)")
    if not all(p.shape == points[0].shape for p in points[1:ndim]):
        raise ValueError("point arrays must share a shape")
    if source.shape[0] != points[0].shape[0]:
        raise ValueError("source and points disagree on n_tot")
    if nufft_type == 3:
        if source.ndim != 3:
            raise ValueError("type-3 source must be (n_tot, n_transf, M)")
        if not all(p.shape == points[ndim].shape for p in points[ndim + 1:]):
            raise ValueError("target arrays must share a shape")
    elif nufft_type == 2:
        if source.ndim != 2 + ndim:
            raise ValueError("type-2 source must be (n_tot, n_transf, N...)")
    else:
        if source.ndim != 3 or source.shape[2] != points[0].shape[1]:
            raise ValueError("type-1 source must be (n_tot, n_transf, M)")
    return single
