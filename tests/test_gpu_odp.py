"""ODPNet (scico/flax/inverse.py:161-462) on the GPU projector, and the
training driver on the GPU.

Values: the gradient-descent network's forward against the same network
run in float64 on the dense matrix of the oracle's float64 projector
(rel l2 <= 1e-4: no CG recurrence amplifies rounding here).  Gradients:
central finite differences along 20 random directions on the float64 twin
(<= 1e-3 of the directional derivative's size), and the float32 GPU
gradients against the twin's (<= 1e-4).  Training: a short run of each
unrolled network through train.BasicTrainer lowers the training loss
(by a fifth or more in 30 steps)."""

import numpy as np
import pytest
import torch

from scico_gb300 import inverse, linop, train, workloads
from test_gpu_inverse import DenseOp, _fd_check, _op

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _no_tf32():
    old = (torch.backends.cudnn.allow_tf32, torch.backends.cuda.matmul.allow_tf32)
    torch.backends.cudnn.allow_tf32 = False
    torch.backends.cuda.matmul.allow_tf32 = False
    yield
    torch.backends.cudnn.allow_tf32, torch.backends.cuda.matmul.allow_tf32 = old


def _case(cuda, n=24, nv=16, batch=3):
    H, g = _op(n=n, nv=nv)
    x_gt = torch.from_numpy(np.stack([workloads.random_ellipses(n, 4, s) for s in range(batch)])).to(cuda)
    return H, g, x_gt, H.project(x_gt)


def _odp(op, depth=3, alpha=0.05, block=inverse.ODPGrDescBlock):
    torch.manual_seed(7)
    return inverse.ODPNet(op, depth=depth, channels=1, num_filters=4, block_depth=2, alpha_ini=alpha,
                          odp_block=block)


def test_odp_forward_vs_dense_twin(cuda):
    H, g, x_gt, y = _case(cuda)
    net = _odp(H).to(cuda).eval()
    out = net(y).detach()
    twin = _odp(DenseOp(H, g, cuda)).to(cuda).double().eval()
    twin.load_state_dict(net.state_dict())
    ref = twin(y.double()).detach()
    rel = float((out.double() - ref).norm() / ref.norm())
    assert rel <= 1e-4, rel
    # alphas start at alpha_ini and halve block by block
    assert [float(b.alpha.detach()) for b in net.blocks] == pytest.approx([0.05, 0.025, 0.0125])


def test_odp_gradients(cuda):
    H, g, x_gt, y = _case(cuda)
    twin = _odp(DenseOp(H, g, cuda)).to(cuda).double()
    yd, xd = y.double(), x_gt.double()
    assert _fd_check(lambda: ((twin(yd) - xd) ** 2).mean(), list(twin.parameters()), eps=1e-6) <= 1e-3
    net = _odp(H).to(cuda)
    twin.load_state_dict(net.state_dict())
    params = list(net.parameters())
    grads = torch.autograd.grad(((net(y).double() - xd) ** 2).mean(), params)
    tg = torch.autograd.grad(((twin(yd) - xd) ** 2).mean(), list(twin.parameters()))
    num = sum(((a.double() - b) ** 2).sum() for a, b in zip(grads, tg)).sqrt()
    den = sum((b ** 2).sum() for b in tg).sqrt()
    assert (num / den).item() <= 1e-4


def test_odp_denoise_block(cuda):
    """ODPProxDnBlock: (ResNet(x) + alpha y) / (1 + alpha), identity operator."""
    torch.manual_seed(3)
    blk = inverse.ODPProxDnBlock(None, depth=2, channels=1, num_filters=4, alpha_ini=0.3).to(cuda).eval()
    x = torch.rand((2, 16, 16), device=cuda)
    y = torch.rand((2, 16, 16), device=cuda)
    want = (blk.resnet(x.unsqueeze(1)).squeeze(1) + 0.3 * y) / 1.3
    assert torch.allclose(blk(x, y), want, rtol=1e-6, atol=1e-6)
    net = inverse.ODPNet(None, depth=2, channels=1, num_filters=4, block_depth=2).to(cuda)
    assert net(y).shape == y.shape


def _ct_data(H, count, seed):
    x = np.stack([workloads.random_ellipses(H.input_shape[0], 6, seed * 100 + k) for k in range(count)])
    y = H.project(torch.from_numpy(x).cuda())
    y = y + 0.01 * y.abs().max() * torch.randn(y.shape, generator=torch.Generator().manual_seed(seed)).cuda()
    return {"image": y.cpu().numpy()[..., None], "label": x[..., None]}


@pytest.mark.parametrize("kind", ["odp", "modl"])
def test_training_run_lowers_loss(cuda, kind):
    """The structure of the reference's CT training scripts (45 views,
    normalized projector 1/N A, ADAM, clip of the learned fidelity weights)
    at a small size: 24 training images of 64^2, 8 test images, 10 epochs."""
    n = 64
    H = linop.XRayTransform2D((n, n), np.linspace(0, np.pi, 45, endpoint=False),
                              det_count=int(n * 1.05 / np.sqrt(2.0)), dx=1.0 / np.sqrt(2))
    Hn = (1.0 / n) * H
    torch.manual_seed(1234)
    if kind == "odp":
        net = inverse.ODPNet(Hn, depth=3, channels=1, num_filters=8, block_depth=3, alpha_ini=1e-2,
                             odp_block=inverse.ODPGrDescBlock)
        post = lambda m: train.clip_positive(m, ("alpha",), minval=1e-3)
    else:
        net = inverse.MoDLNet(Hn, depth=2, channels=1, num_filters=8, block_depth=3, lmbda_ini=0.5, cg_iter=4)
        post = lambda m: train.clip_positive(m, ("lmbda",), minval=5e-4)
    cfg = {"seed": 1234, "opt_type": "ADAM", "batch_size": 8, "num_epochs": 10, "base_learning_rate": 1e-3,
           "log_every_steps": 6, "post_lst": [post]}
    tr = train.BasicTrainer(cfg, net, _ct_data(Hn, 24, 1), _ct_data(Hn, 8, 2))
    _, stats = tr.train()
    assert tr.num_steps == 30 and len(stats) == 5
    assert stats[-1]["Train_Loss"] < 0.8 * stats[0]["Train_Loss"], [r["Train_Loss"] for r in stats]
    assert all(np.isfinite(r["Eval_SNR"]) for r in stats)
