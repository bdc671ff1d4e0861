"""fr_resolve_async / fr_resolve_wait: the image copied while the next
iteration runs is the image of the state it was queued on."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_async_resolve_matches_sync_and_overlaps():
    import torch
    from frsppm import abi, scenes
    sc = scenes.cornell_box(width=32, height=32)
    n = 32 * 32
    bufs = [torch.empty((n, 4), dtype=torch.float32, pin_memory=True) for _ in range(3)]
    with abi.Renderer(sc, 2000, alpha=0.9, radius=0.015) as r, abi.Renderer(sc, 2000, alpha=0.9, radius=0.015) as twin:
        r.iterate(1)
        t = r.resolve_async(bufs[0].data_ptr())
        r.resolve_wait(t)
        np.testing.assert_array_equal(bufs[0].numpy(), r.resolve())   # same state: the same image
        images = []
        for k in range(3):  # queue each resolve, run the next iteration, then wait
            r.iterate(1, sync=False)
            t = r.resolve_async(bufs[k].data_ptr())
            r.iterate(1, sync=False)
            r.resolve_wait(t)
            images.append(bufs[k].numpy().copy())
        r.synchronize()
        # The twin, resolved synchronously after the same iteration counts
        # (2, 4, 6 iterations in): equal up to the float rounding of the grid
        # cells' atomic slot order.
        for k in range(3):
            twin.iterate(2)
            ref = twin.resolve()
            assert np.abs(images[k] - ref).max() <= 1e-5 * np.abs(ref).max()
        assert not np.array_equal(images[0], images[1])
    with pytest.raises(RuntimeError):
        with abi.Renderer(sc, 2000) as r:
            r.resolve_wait(5)   # no such ticket
