"""Bounded waits of the bin scan, made to run out without faulting anything.

The scan chains its tiles of 1024 bins through a look-back in which a tile
waits, with a bound, for its predecessors to publish.  `gbr_set_scan_wait`
(a test hook) makes one tile publish nothing and lowers the bound, so the
tiles after it give up.  The frame must then be reported as GBR_ERR_TIMEOUT
-- its fill, raster and shade kernels return before they read an offset, so
nothing is written past the bin storage -- and the next frame, with the
hook cleared, must render exactly as before.  Covers exact binning's scan
and the capacity scan of predicted binning.
"""
import ctypes as C

import numpy as np
import pytest

import scenes
from oracle import mlp_oracle

pytestmark = pytest.mark.gpu


def _outputs(r):
    colour, depth = r.readback()
    ids = r.readback_ids()
    offsets, bins = r.get_bins()
    return colour.copy(), depth.copy(), ids.copy(), offsets.copy(), bins.copy()


def _assert_same(a, b):
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("silent_tile,waited_on", [(0, True), (2, True), (4, False)])
def test_scan_wait_runs_out_and_the_frame_is_flagged(gbr_lib, cuda_device, silent_tile, waited_on):
    """Tiles 0 and 2 have successors that wait for them: the frame is
    flagged.  Tile 4 is the last of the 5: nothing waits for it, it still
    computes its own prefix and the frame's totals, and the frame is valid."""
    import torch
    # 640x480 with 8x8 bins: 4,800 bins, 5 scan tiles
    s = scenes.soup_scene(40_000, 640, 480, 8, seed=17)
    with gbr_lib.Renderer(s.width, s.height) as r:
        r.load_scene(s, 256)
        r.render_scene(s)
        good = _outputs(r)
        r.set_scan_wait(spin_limit=64, silent_tile=silent_tile)
        r.render_scene(s)
        if not waited_on:
            _assert_same(good, _outputs(r))
            return
        with pytest.raises(gbr_lib.GbrError) as e:
            r.readback()
        assert e.value.status == 4, str(e.value)   # GBR_ERR_TIMEOUT
        with pytest.raises(gbr_lib.GbrError) as e:
            r.stats()
        assert e.value.status == 4
        torch.cuda.synchronize()   # the context is intact
        r.set_scan_wait(0, -1)
        r.render_scene(s)
        _assert_same(good, _outputs(r))
        # a second frame reuses the restarted scan state
        r.render_scene(s)
        _assert_same(good, _outputs(r))


def test_capacity_scan_wait_runs_out_under_predicted_binning(gbr_lib, cuda_device):
    s = scenes.soup_scene(40_000, 640, 480, 8, seed=23)
    w = np.zeros(mlp_oracle.NUM_PARAMS, np.float32)
    w[mlp_oracle.OFF_B3] = 60.0   # every bin predicted to hold ~60 entries
    w16 = mlp_oracle.f32_to_bf16(w)
    with gbr_lib.Renderer(s.width, s.height) as r:
        r.load_scene(s, 256)
        r.render_scene(s)
        good = _outputs(r)
        gbr_lib.check(r._lib.gbr_set_predictor(r.h, w16.ctypes.data_as(C.c_void_p), len(w16), C.c_float(0.0),
                                               C.c_float(0.0), C.c_float(0.0)))
        r.set_binning(gbr_lib.BINNING_PREDICTED)
        r.render_scene(s)
        r.stats()
        r.set_scan_wait(spin_limit=64, silent_tile=1)
        r.render_scene(s)
        with pytest.raises(gbr_lib.GbrError) as e:
            r.readback()
        assert e.value.status == 4, str(e.value)
        r.set_scan_wait(0, -1)
        r.render_scene(s)
        _assert_same(good, _outputs(r))
