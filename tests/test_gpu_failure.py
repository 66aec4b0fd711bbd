"""Failure handling without a GPU fault: every spin or traversal loop of the kernels
has an iteration cap; a cap that runs out ends the loop, sets a LUZ_DEV_* bit in the
context's device status word and lets the kernel return, so the context stays usable.
The test lowers the visibility kernel's per-ray step cap through the debug knob (off
by default) so that it runs out on every ray."""
import numpy as np
import pytest

import luz_gb300 as L

pytestmark = pytest.mark.gpu

LUZ_ERR_DEVICE = 4
LUZ_DEV_TRAVERSAL_CAP = 1 << 2


def _lit_bits(frame):
    """The lit pixels as one bit plane (pixel p: bit p & 31 of word p >> 5)."""
    lit = (np.linalg.norm(frame.read(L.PLANE_NORMAL)[..., :3], axis=-1) > 0).reshape(-1)
    p = np.nonzero(lit)[0]
    words = np.zeros((lit.size + 31) // 32, np.uint32)
    np.bitwise_or.at(words, p >> 5, (np.uint32(1) << (p & 31).astype(np.uint32)))
    return words


def test_traversal_step_cap_runs_out_reports_and_recovers():
    ctx = L.Context(0)
    try:
        s = L.HostScene(1, width=128, height=96)
        g = L.GPUScene(ctx, s)
        g.render(0)
        ctx.synchronize()
        assert ctx.device_status() == 0
        ao_ref = g.frame.read(L.PLANE_AO_BITS).copy()
        sh_ref = g.frame.read(L.PLANE_SHADOW_BITS).copy()
        assert sh_ref.any() and (ao_ref != _lit_bits(g.frame)).any()   # some occlusion to lose

        ctx.set_debug_step_cap(4)               # below the steps of one refill round
        g.frame.trace(g.tlas, 0)                # asynchronous: the call itself succeeds
        with pytest.raises(L.LuzError) as e:
            ctx.synchronize()                   # the kernel returned; its status is reported
        assert e.value.status == LUZ_ERR_DEVICE
        assert ctx.device_status() & LUZ_DEV_TRAVERSAL_CAP   # read and cleared
        # every ray ended at once: no shadow hit recorded, every AO sample a miss
        assert not g.frame.read(L.PLANE_SHADOW_BITS).any()
        lit = _lit_bits(g.frame)
        assert np.array_equal(g.frame.read(L.PLANE_AO_BITS) & lit, np.broadcast_to(lit, ao_ref.shape))

        ctx.set_debug_step_cap(0)               # the library's cap again: same masks as before
        g.frame.trace(g.tlas, 0)
        ctx.synchronize()
        assert ctx.device_status() == 0
        assert np.array_equal(g.frame.read(L.PLANE_AO_BITS), ao_ref)
        assert np.array_equal(g.frame.read(L.PLANE_SHADOW_BITS), sh_ref)
    finally:
        ctx.close()
