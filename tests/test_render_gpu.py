"""Headless splat rasteriser against the oracle's sequential restatement of the reference's background and
blend (libs/render/source/cuda-render.cu:214-310): the device image equals the oracle's byte for byte."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _raster(gpe_mod, torch, width, height, scale, chunk_dim, pad=64):
    pitch = 4 * width + pad
    img = torch.zeros((height, pitch), dtype=torch.uint8, device="cuda")
    cov = torch.zeros((height, width), dtype=torch.int32, device="cuda")
    r = gpe_mod.Raster(img.data_ptr(), pitch, width, height, scale, chunk_dim, cov.data_ptr())
    return r, img, cov


def _view_from(gpe_mod, torch, pos, counts, chunks_x, chunks_y, chunk_dim, cap):
    p = torch.from_numpy(np.ascontiguousarray(pos, np.float32)).cuda()
    v = torch.zeros_like(p)
    c = torch.from_numpy(np.ascontiguousarray(counts, np.int32)).cuda()
    view = gpe_mod.View(p.data_ptr(), v.data_ptr(), c.data_ptr(), chunks_x, chunks_y, chunk_dim, cap)
    return view, (p, v, c)


@pytest.mark.parametrize("seed", [0, 1])
def test_render_matches_oracle_random_view(gpe_mod, cuda_ok, oracle, seed):
    torch = pytest.importorskip("torch")
    g = np.random.default_rng(seed)
    cx, cy, dim, cap = 12, 6, 32.0, 1536  # the reference's world (constants.h:11-12, 48-50)
    counts = g.integers(0, cap + 200, cx * cy).astype(np.int32)  # some chunks over capacity: clipped
    pos = np.empty((cx * cy, cap, 2), np.float32)
    for c in range(cx * cy):
        ox, oy = (c % cx) * dim, (c // cx) * dim
        pos[c, :, 0] = ox + g.uniform(-2, dim + 2, cap)  # some atoms just outside the image
        pos[c, :, 1] = oy + g.uniform(-2, dim + 2, cap)
    view, keep = _view_from(gpe_mod, torch, pos.reshape(-1, 2), counts, cx, cy, dim, cap)
    W, H, scale = int(cx * dim * 5), int(cy * dim * 5), 5.0  # kDispWidth x kDispHeight
    r, img, cov = _raster(gpe_mod, torch, W, H, scale, dim)
    gpe_mod.render_frame(r, view)
    torch.cuda.synchronize()
    got = img[:, : 4 * W].cpu().numpy().reshape(H, W, 4)
    want = oracle.render_frame(W, H, scale, dim, pos, counts)
    diff = np.argwhere(got != want)
    assert len(diff) == 0, (len(diff), diff[:5])
    assert cov.sum().item() > 0


def test_render_published_pbf_frame(gpe_mod, cuda_ok, oracle):
    """A PBF step published into a view (gpe_pbf_publish) and drawn: the same bytes as the oracle."""
    torch = pytest.importorskip("torch")
    from gpe import scenes

    p = scenes.reference_pbf_params(iters=2)
    pos, vel, boxes = scenes.reference_pbf_block()
    e = gpe_mod.Pbf(p, boxes, capacity=len(pos))
    e.set_state(pos, vel)
    e.step(5)
    cx, cy, dim, cap = 12, 6, 32.0, 1536
    vp = torch.zeros((cx * cy * cap, 2), dtype=torch.float32, device="cuda")
    vv = torch.zeros_like(vp)
    vc = torch.zeros(cx * cy, dtype=torch.int32, device="cuda")
    view = gpe_mod.View(vp.data_ptr(), vv.data_ptr(), vc.data_ptr(), cx, cy, dim, cap)
    e.publish(view)
    W, H = int(cx * dim * 5), int(cy * dim * 5)
    r, img, _ = _raster(gpe_mod, torch, W, H, 5.0, dim, pad=0)
    gpe_mod.render_frame(r, view)
    torch.cuda.synchronize()
    got = img.cpu().numpy().reshape(H, W, 4)
    want = oracle.render_frame(W, H, 5.0, dim, vp.cpu().numpy().reshape(cx * cy, cap, 2), vc.cpu().numpy())
    np.testing.assert_array_equal(got, want)
    # the splats changed the picture where the fluid is
    assert (got[..., 2] != 80).sum() > len(pos)


def test_render_device_view_captured_with_step_and_publish(gpe_mod, cuda_ok, oracle):
    """enqueue + publish + render_frame recorded into one CUDA graph with the view struct in device memory
    (read only by the kernels), replayed twice: each replay's image equals the oracle's drawing of the view
    that replay published."""
    torch = pytest.importorskip("torch")
    import ctypes as C

    from gpe import scenes

    p = scenes.reference_pbf_params(iters=2)
    pos, vel, boxes = scenes.reference_pbf_block()
    e = gpe_mod.Pbf(p, boxes, capacity=len(pos))
    e.set_state(pos, vel)
    cx, cy, dim, cap = 12, 6, 32.0, 1536
    vp = torch.zeros((cx * cy * cap, 2), dtype=torch.float32, device="cuda")
    vv = torch.zeros_like(vp)
    vc = torch.zeros(cx * cy, dtype=torch.int32, device="cuda")
    view = gpe_mod.View(vp.data_ptr(), vv.data_ptr(), vc.data_ptr(), cx, cy, dim, cap)
    raw = bytes(C.string_at(C.addressof(view), C.sizeof(view)))
    dview = torch.frombuffer(bytearray(raw), dtype=torch.uint8).cuda()
    W, H = int(cx * dim * 5), int(cy * dim * 5)
    r, img, _ = _raster(gpe_mod, torch, W, H, 5.0, dim, pad=0)
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.graph(g, stream=s):
        st = torch.cuda.current_stream().cuda_stream
        e.enqueue(3, stream=st)
        e.publish(dview.data_ptr(), view_mem=gpe_mod.MEM_DEVICE, stream=st)
        gpe_mod.render_frame(r, dview.data_ptr(), view_mem=gpe_mod.MEM_DEVICE, stream=st)
    for _ in range(2):
        g.replay()
        torch.cuda.synchronize()
        got = img.cpu().numpy().reshape(H, W, 4)
        want = oracle.render_frame(W, H, 5.0, dim, vp.cpu().numpy().reshape(cx * cy, cap, 2), vc.cpu().numpy())
        np.testing.assert_array_equal(got, want)
