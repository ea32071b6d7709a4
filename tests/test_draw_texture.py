"""DrawTexture / DrawTextureGlobal (CUDARenderer.cu:1968-2012) through the C
ABI: the texture-hardware blit against exact texel indices, the
software-sampler blit against the oracle's sampler, every pixel."""
import numpy as np
import pytest

from oracle import oracle

W, H = 160, 120


def texture(w, h, seed):
    rng = np.random.default_rng(seed)
    return rng.integers(0, 2**32, size=(h, w), dtype=np.uint64).astype(np.uint32)


@pytest.mark.gpu
@pytest.mark.parametrize("tw, th", [(97, 61), (64, 32), (320, 240)])
def test_draw_texture_hardware_blit(gbr_lib, cuda_device, tw, th):
    """Texel (floor(x*tw/W), floor(y*th/H)) with red and blue swapped; pixels
    whose texel coordinate lies within 1/64 texel of a texel edge are left to
    the texture unit's coordinate rounding and only counted (97-texel rows
    are not pitch-aligned: the reader's pitched copy is used)."""
    tex = texture(tw, th, tw)
    with gbr_lib.Renderer(W, H) as r:
        tid = r.add_texture(tex)
        r.draw_texture(tid)
        colour, _ = r.readback()
    x = np.arange(W)
    y = np.arange(H)
    tx, fx = np.divmod(x * tw, W)
    ty, fy = np.divmod(y * th, H)
    t = tex[ty[:, None], tx[None, :]]
    want = (t & 0xFF00FF00) | ((t & 0xFF) << 16) | ((t >> 16) & 0xFF)
    edge_x = (fx < W / 64) | (fx > W - W / 64)
    edge_y = (fy < H / 64) | (fy > H - H / 64)
    clear = ~(edge_x[None, :] | edge_y[:, None])
    assert np.array_equal(colour[clear], want[clear])
    # at texel edges the result is still one of the two neighbouring texels
    tx1 = np.minimum(tx + 1, tw - 1)
    txm = np.maximum(tx - 1, 0)
    ok = np.zeros((H, W), bool)
    for yy in (np.maximum(ty - 1, 0), ty, np.minimum(ty + 1, th - 1)):
        for xx in (txm, tx, tx1):
            tt = tex[yy[:, None], xx[None, :]]
            ok |= colour == ((tt & 0xFF00FF00) | ((tt & 0xFF) << 16) | ((tt >> 16) & 0xFF))
    assert ok.all()


@pytest.mark.gpu
@pytest.mark.parametrize("stretch", [True, False])
@pytest.mark.parametrize("sample", [0, 1])
def test_draw_texture_global_matches_oracle_sampler(gbr_lib, cuda_device, stretch, sample):
    tex = texture(96, 72, 3 + sample)
    with gbr_lib.Renderer(W, H) as r:
        tid = r.add_texture(tex)
        r.draw_texture_global(tid, stretch, sample)
        colour, _ = r.readback()
    dw, dh = (W, H) if stretch else tex.shape[::-1]
    want = np.empty((H, W), np.uint32)
    for yy in range(H):
        v = np.float32(yy) / np.float32(dh)
        for xx in range(W):
            u = np.float32(xx) / np.float32(dw)
            want[yy, xx] = oracle.rgba_from_colour(oracle.sample(tex, float(u), float(v), sample))
    assert np.array_equal(colour, want)
    if not stretch:   # past the texture: the sampler's magenta
        assert colour[0, W - 1] == oracle.rgba_from_colour((1.0, 0.0, 1.0))


@pytest.mark.gpu
def test_draw_texture_errors(gbr_lib, cuda_device):
    with gbr_lib.Renderer(W, H) as r:
        with pytest.raises(gbr_lib.GbrError) as e:
            r.draw_texture(3)
        assert e.value.status == 6
        tid = r.add_texture(texture(8, 8, 1))
        with pytest.raises(gbr_lib.GbrError) as e:
            r.draw_texture_global(tid, True, 7)
        assert e.value.status == 1
        r.remove_texture(tid)
        with pytest.raises(gbr_lib.GbrError):
            r.draw_texture(tid)
