"""RaggedBatch packing (host logic, no GPU)."""

import pytest
import torch

from torchmorph_gb300 import RaggedBatch


def test_pack_and_views():
    a = torch.arange(6.0).reshape(2, 3)
    b = torch.arange(4.0).reshape(1, 1, 4, 1)
    rb = RaggedBatch.from_images([a, b])
    assert rb.shapes == [(2, 3), (4, 1)] and rb.offsets == [0, 6] and rb.numel == 10
    assert torch.equal(rb[0], a) and torch.equal(rb[1], b[0, 0])
    m = rb.map(lambda x: x > 2)
    assert m.dtype == torch.bool and m.shapes == rb.shapes
    assert torch.equal(m[0], a > 2)


def test_custom_offsets_and_errors():
    data = torch.zeros(20)
    rb = RaggedBatch(data, [(2, 2), (3, 3)], offsets=[10, 0])
    assert rb[0].shape == (2, 2) and rb[0].data_ptr() == data[10:].data_ptr()
    with pytest.raises(ValueError, match="outside"):
        RaggedBatch(data, [(5, 5)])
    with pytest.raises(ValueError, match="non-empty"):
        RaggedBatch(data, [(0, 5)])
    with pytest.raises(ValueError, match="at least one"):
        RaggedBatch.from_images([])
    with pytest.raises(ValueError, match="CUDA"):
        _ = rb.plan


def test_volumes_pack_and_dimension_errors():
    a = torch.arange(24.0).reshape(2, 3, 4)
    b = torch.arange(5.0).reshape(1, 1, 1, 5, 1)
    rb = RaggedBatch.from_images([a, b])
    assert rb.ndim == 3 and rb.shapes == [(2, 3, 4), (1, 5, 1)] and rb.offsets == [0, 24] and rb.numel == 29
    assert torch.equal(rb[0], a) and torch.equal(rb[1], b[0, 0])
    with pytest.raises(ValueError, match="all be 2-D or all be 3-D"):
        RaggedBatch(torch.zeros(40), [(2, 3), (2, 2, 2)])
    with pytest.raises(ValueError, match=r"\(D, H, W\)"):
        RaggedBatch.from_images([torch.zeros(2, 2, 2, 2)])
    from torchmorph_gb300 import ragged
    with pytest.raises(ValueError, match="CUDA"):
        ragged.euclidean_distance_transform(rb)
