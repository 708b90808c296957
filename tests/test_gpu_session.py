"""RenderSession: the preallocated, sync-free forward+backward (device-side
intersection count, capacity-sized buffers), eager and as a CUDA graph."""

import numpy as np
import pytest

from conftest import GRAD_RTOL, IMG_ATOL, normwise_rel

pytestmark = pytest.mark.gpu


def _scene():
    from jaxsplat_gb300.scenes import make_scene

    return make_scene("small", seed=21, num_points=30_000, img_shape=(160, 224))


def _session(sc, capacity=None):
    from jaxsplat_gb300.session import RenderSession

    kw = sc.kwargs
    s = RenderSession(sc.spec.num_points, img_shape=kw["img_shape"], f=kw["f"], c=kw["c"],
                      glob_scale=kw["glob_scale"], clip_thresh=kw["clip_thresh"],
                      block_size=16, capacity=capacity)
    s.set_inputs(sc.means3d, sc.scales, sc.quats, sc.colors, sc.opacities, sc.viewmat,
                 sc.background, sc.target)
    return s


def test_session_matches_autograd_render_and_graph_replay():
    import torch

    import jaxsplat_gb300 as js

    sc = _scene()
    sess = _session(sc)
    count = sess.measure_capacity()
    assert sess.capacity > count
    sess.step()
    eager = {k: v.clone() for k, v in sess.grads.items()}
    eager_img = sess.img.clone()
    eager_loss = float(sess.loss.item())
    assert sess.check() == count

    sess.capture()
    sess.replay()
    sess.replay()
    assert sess.check() == count
    torch.testing.assert_close(sess.img, eager_img, rtol=0, atol=0)
    for k, v in sess.grads.items():
        assert normwise_rel(v.cpu().numpy(), eager[k].cpu().numpy()) <= 1e-5, k

    t = {k: torch.from_numpy(getattr(sc, k)).cuda()
         for k in ("means3d", "scales", "quats", "colors", "opacities", "viewmat", "background",
                   "target")}
    for k in ("means3d", "scales", "quats", "colors", "opacities"):
        t[k].requires_grad_(True)
    img = js.render(t["means3d"], t["scales"], t["quats"], t["colors"], t["opacities"],
                    viewmat=t["viewmat"], background=t["background"], block_size=16, **sc.kwargs)
    loss = torch.mean((img - t["target"]) ** 2)
    loss.backward()
    assert float(np.abs(img.detach().cpu().numpy() - eager_img.cpu().numpy()).max()) <= IMG_ATOL
    assert abs(float(loss.item()) - eager_loss) <= 1e-6 * max(1.0, abs(eager_loss))
    for k in ("means3d", "scales", "quats", "colors", "opacities"):
        assert normwise_rel(eager[k].cpu().numpy(), t[k].grad.cpu().numpy()) <= GRAD_RTOL, k


def test_device_count_sort_matches_exact_count():
    import torch

    from jaxsplat_gb300 import _ops

    sc = _scene()
    sess = _session(sc)
    count = sess.measure_capacity()
    sess.step()
    sess.check()
    kw = dict(img_shape=sc.kwargs["img_shape"], block_width=16)
    exact = _ops.sort_and_bin(count, sess.xys, sess.depths, sess.radii, sess.cum, **kw)
    torch.testing.assert_close(sess.ids_sorted[:count], exact["gaussian_ids_sorted"], rtol=0, atol=0)
    torch.testing.assert_close(sess.tile_bins, exact["tile_bins"], rtol=0, atol=0)


def test_capacity_overflow_is_reported():
    from jaxsplat_gb300._lib import SplatError

    sc = _scene()
    sess = _session(sc, capacity=1000)
    sess.step()
    with pytest.raises(SplatError, match="capacity-exceeded"):
        sess.check()


def test_step_io_copies_inputs_in_and_results_out():
    """step_io / its graph: the host input block reaches the device (a changed
    target changes the loss), and the host output block holds the same loss
    and gradients as a device step on those inputs."""
    import torch

    sc = _scene()
    sess = _session(sc)
    sess.measure_capacity()
    target_b = (sc.target * 0.5 + 0.25).astype(np.float32)
    host_in = sess.host_inputs(sc.means3d, sc.scales, sc.quats, sc.colors, sc.opacities,
                               sc.viewmat, sc.background, target_b)
    host_out = torch.empty(sess.outputs.numel(), dtype=torch.float32, pin_memory=True)
    sess.capture_io(host_in, host_out)
    host_out.fill_(float("nan"))
    sess.replay_io()
    torch.cuda.synchronize()
    got = host_out.clone()
    sess.step()  # same (uploaded) inputs, device only
    torch.cuda.synchronize()
    ref = sess.outputs.cpu()
    assert abs(float(got[0]) - float(ref[0])) <= 1e-6 * max(1.0, abs(float(ref[0])))
    assert normwise_rel(got.numpy(), ref.numpy()) <= 1e-5
    torch.testing.assert_close(sess.target.cpu(), torch.from_numpy(target_b), rtol=0, atol=0)


def test_stream_step_matches_step_io_for_each_input():
    """stream_step (double-buffered, copies overlapped across steps): four
    consecutive steps alternating two input sets each return the loss and
    gradients that step_io gives for that input set."""
    import torch

    sc = _scene()
    sess = _session(sc)
    sess.measure_capacity()
    targets = [sc.target, (sc.target * 0.5 + 0.25).astype(np.float32)]
    scales = [sc.scales, (sc.scales * 1.1).astype(np.float32)]
    host_in = [sess.host_inputs(sc.means3d, scales[j], sc.quats, sc.colors, sc.opacities,
                                sc.viewmat, sc.background, targets[j]) for j in range(2)]
    n_out = sess.outputs.numel()
    refs = []
    for j in range(2):
        out = torch.empty(n_out, dtype=torch.float32, pin_memory=True)
        sess.step_io(host_in[j], out)
        torch.cuda.synchronize()
        refs.append(out.clone())
    assert float(refs[0][0]) != float(refs[1][0])
    outs = [torch.full((n_out,), float("nan"), pin_memory=True) for _ in range(4)]
    for i in range(4):
        sess.stream_step(host_in[i % 2], outs[i])
    sess.stream_sync()
    torch.cuda.synchronize()
    for i in range(4):
        ref = refs[i % 2]
        assert abs(float(outs[i][0]) - float(ref[0])) <= 1e-6 * max(1.0, abs(float(ref[0]))), i
        assert normwise_rel(outs[i].numpy(), ref.numpy()) <= 1e-5, i
