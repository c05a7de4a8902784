"""The CUDA U-Net (bf16 tensor-core convolutions, FP32 accumulate) against the
FP64 oracle of oracle/unet_oracle.py on the same bf16-rounded weights and
inputs.  Bar (bf16 activations): forward relative L2 <= 3e-2; every layer's
weight gradient relative L2 <= 8e-2 and cosine >= 0.995 against FP64."""
import numpy as np
import pytest

from oracle import unet_oracle as U

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

H, W, WIDTHS, N = 16, 32, (16, 32, 32, 48), 2


def bf16_round(a):
    t = torch.tensor(np.asarray(a, dtype=np.float32)).to(torch.bfloat16)
    return t.to(torch.float32).numpy().astype(np.float64)


def _net(kind=None, h=H, w=W, n=N):
    from lbm_mirror_gb300 import UNet
    net = UNet(height=h, width=w, widths=WIDTHS, out_channels=3, max_batch=n, seed=7)
    if kind is not None:
        net.set_conv_kernel(kind)
    return net


KINDS = [pytest.param(0, id="tcgen05"), pytest.param(1, id="mma_sync")]


def _inputs(rng, h=H, w=W, n=N):
    x = np.zeros((n, h, w, 16))
    x[..., :3] = rng.standard_normal((n, h, w, 3))
    return bf16_round(x)


# 16 x 32: every level below 128 pixels wide (per-tile kernels); 8 x 128: the
# full-resolution level through the row-run convolution and the halo weight
# gradient, the 64-pixel level through the halo weight gradient with 64-pixel
# row tiles
SHAPES = [pytest.param((H, W, N), id="16x32"), pytest.param((8, 128, 1), id="8x128")]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("kind", KINDS)
def test_forward_and_gradients_vs_fp64_oracle(kind, shape):
    h, w, n = shape
    rng = np.random.default_rng(1)
    net = _net(kind, h, w, n)
    flat = net.params().astype(np.float64)
    assert flat.size == U.param_count(16, 3, WIDTHS)
    x = _inputs(rng, h, w, n)
    tgt = rng.standard_normal((n, h, w, 3)) * 0.1
    xin = torch.tensor(x, dtype=torch.bfloat16, device="cuda").contiguous()
    tg = torch.tensor(tgt, dtype=torch.float32, device="cuda").contiguous()
    out = torch.empty((n, h, w, 3), dtype=torch.float32, device="cuda")
    net.set_input(xin.data_ptr(), n)
    net.forward(n, out.data_ptr())
    loss_gpu = net.backward(tg.data_ptr(), n)
    net.synchronize()
    g_gpu = net.grads().astype(np.float64)

    # oracle on bf16 conv weights (what the tensor cores multiply); biases and
    # the 1x1 head stay FP32 on the GPU
    shapes = U.layer_shapes(16, 3, WIDTHS)
    wq = flat.copy()
    o = 0
    for (name, co, k, ci) in shapes:
        nw = co * k * k * ci
        if k == 3:
            wq[o:o + nw] = bf16_round(flat[o:o + nw])
        o += nw + co
    loss, y, g = U.loss_and_grads(wq, x, tgt, 16, 3, WIDTHS)
    y_gpu = out.cpu().numpy().astype(np.float64)
    assert np.linalg.norm(y_gpu - y) / np.linalg.norm(y) <= 3e-2
    assert abs(loss_gpu - loss) <= 3e-2 * loss
    o = 0
    for (name, co, k, ci) in shapes:
        nw = co * k * k * ci
        for sl in (slice(o, o + nw), slice(o + nw, o + nw + co)):
            a, b = g_gpu[sl], g[sl]
            rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
            cos = a @ b / max(np.linalg.norm(a) * np.linalg.norm(b), 1e-30)
            assert rel <= 8e-2 and cos >= 0.995, (name, rel, cos)
        o += nw + co


def test_training_reduces_loss():
    rng = np.random.default_rng(2)
    net = _net()
    x = _inputs(rng)
    # a smooth target the net can fit: a function of the input planes
    tgt = np.stack([np.tanh(x[..., 0]), 0.5 * x[..., 1], 0.1 * x[..., 0] * x[..., 2]], axis=-1)
    xin = torch.tensor(x, dtype=torch.bfloat16, device="cuda").contiguous()
    tg = torch.tensor(tgt, dtype=torch.float32, device="cuda").contiguous()
    net.set_input(xin.data_ptr(), N)
    losses = []
    for _ in range(150):
        net.forward(N)
        losses.append(net.backward(tg.data_ptr(), N))
        net.adam_step(lr=3e-3)
    assert losses[-1] < 0.2 * losses[0], (losses[0], losses[-1])
    assert np.isfinite(losses).all()


def test_tcgen05_and_mma_sync_kernels_agree_at_full_size():
    """The 256x64 warm-start network (widths 32, 64, 128, 128: data-gradient
    GEMMs with N = 32 .. 256) at the training batch of 32 through both
    convolution kernels on the same weights and inputs: outputs and every
    gradient agree to bf16 rounding of the activations (relative L2 <= 1e-2).
    At this batch the tcgen05 path takes its production shapes (row-run
    convolutions, multi-row halo tiles, halo weight gradients)."""
    from lbm_mirror_gb300 import UNet
    rng = np.random.default_rng(9)
    n, h, w = 32, 64, 256
    x = np.zeros((n, h, w, 16), np.float32)
    x[..., :3] = rng.standard_normal((n, h, w, 3))
    tgt = 0.1 * rng.standard_normal((n, h, w, 3)).astype(np.float32)
    xin = torch.tensor(x, dtype=torch.bfloat16, device="cuda").contiguous()
    tg = torch.tensor(tgt, device="cuda").contiguous()
    res = {}
    for kind in (0, 1):
        net = UNet(height=h, width=w, widths=(32, 64, 128, 128), out_channels=3, max_batch=n, seed=3)
        net.set_conv_kernel(kind)
        out = torch.empty((n, h, w, 3), dtype=torch.float32, device="cuda")
        net.set_input(xin.data_ptr(), n)
        net.forward(n, out.data_ptr())
        loss = net.backward(tg.data_ptr(), n)
        net.synchronize()
        res[kind] = (out.cpu().numpy().astype(np.float64), net.grads().astype(np.float64), loss)
    (ya, ga, la), (yb, gb, lb) = res[0], res[1]
    assert np.linalg.norm(ya - yb) / np.linalg.norm(yb) <= 1e-2
    assert abs(la - lb) <= 1e-2 * lb
    assert np.linalg.norm(ga - gb) / np.linalg.norm(gb) <= 1e-2



def test_residual_head_adds_the_input_plane():
    """kel_unet_set_residual: output channel 0 = the plain head + 2 x input
    plane 9 (the warm start's local Poiseuille estimate); the other output
    channels and the gradients' path are unchanged; out_channel -1 turns it
    off; out-of-range channels are rejected."""
    from lbm_mirror_gb300 import KelError
    rng = np.random.default_rng(4)
    net = _net()
    x = np.zeros((N, H, W, 16))
    x[..., :3] = rng.standard_normal((N, H, W, 3))
    x[..., 9] = rng.uniform(0.0, 4.0, (N, H, W))
    x = bf16_round(x)
    xin = torch.tensor(x, dtype=torch.bfloat16, device="cuda").contiguous()
    base = torch.empty((N, H, W, 3), dtype=torch.float32, device="cuda")
    res = torch.empty_like(base)
    net.set_input(xin.data_ptr(), N)
    net.forward(N, base.data_ptr())
    net.set_residual(0, 9, 2.0)
    net.forward(N, res.data_ptr())
    net.synchronize()
    b, r = base.cpu().numpy(), res.cpu().numpy()
    np.testing.assert_allclose(r[..., 0], b[..., 0] + 2.0 * x[..., 9], rtol=0, atol=1e-5)
    np.testing.assert_array_equal(r[..., 1:], b[..., 1:])
    net.set_residual(-1)
    net.forward(N, res.data_ptr())
    net.synchronize()
    np.testing.assert_array_equal(res.cpu().numpy(), b)
    with pytest.raises(KelError):
        net.set_residual(3, 9, 1.0)
    with pytest.raises(KelError):
        net.set_residual(0, 16, 1.0)


def test_train_step_graph_equals_separate_calls():
    """kel_unet_train_step (first step launched one by one, then a captured
    graph replayed) against forward + backward + adam_step: the same
    parameters and losses, bit for bit, over five steps with a changing
    learning rate; on a 16x256 grid so that both convolution kernels run."""
    from lbm_mirror_gb300 import UNet
    rng = np.random.default_rng(12)
    n, h, w = 2, 16, 256
    x = np.zeros((n, h, w, 16), np.float32)
    x[..., :3] = rng.standard_normal((n, h, w, 3))
    xin = torch.tensor(x, dtype=torch.bfloat16, device="cuda").contiguous()
    tg = torch.tensor(0.1 * rng.standard_normal((n, h, w, 3)).astype(np.float32), device="cuda").contiguous()
    a = UNet(height=h, width=w, widths=(16, 32, 32, 48), out_channels=3, max_batch=n, seed=4)
    b = UNet(height=h, width=w, widths=(16, 32, 32, 48), out_channels=3, max_batch=n, seed=4)
    torch.cuda.synchronize()
    la = []
    for k in range(5):
        lr = 1e-3 * (k + 1)
        a.set_input(xin.data_ptr(), n)
        a.forward(n)
        la.append(a.backward(tg.data_ptr(), n))
        a.adam_step(lr=lr)
        b.set_input(xin.data_ptr(), n)
        b.train_step(tg.data_ptr(), n, lr=lr)
        assert b.last_loss() == la[-1], (k, b.last_loss(), la[-1])
    a.synchronize()
    b.synchronize()
    assert np.array_equal(a.params(), b.params())
