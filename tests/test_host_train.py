"""The training driver's host logic on CPU (no GPU): learning-rate
schedules against their closed forms (scico/flax/train/learning_rate.py),
loss and SNR definitions, parameter clipping, batching, and a short
training run of ODPNet over a dense toy operator (the loop, post-step
clipping, evaluation, checkpoint and resume)."""

import math

import numpy as np
import pytest
import torch

from scico_gb300 import inverse, train


def test_schedules():
    cfg = {"base_learning_rate": 1e-3, "num_epochs": 10, "steps_per_epoch": 5, "lr_decay_rate": 0.5,
           "warmup_epochs": 2}
    assert train.create_cnst_lr_schedule(cfg)(37) == 1e-3
    ex = train.create_exp_lr_schedule(cfg)
    assert ex(0) == pytest.approx(1e-3) and ex(50) == pytest.approx(5e-4) and ex(25) == pytest.approx(1e-3 * 0.5**0.5)
    co = train.create_cosine_lr_schedule(cfg)
    assert co(0) == 0.0 and co(5) == pytest.approx(5e-4) and co(10) == pytest.approx(1e-3)
    assert co(10 + 20) == pytest.approx(1e-3 * 0.5 * (1 + math.cos(math.pi * 0.5)))
    assert co(10 + 40) == pytest.approx(0.0, abs=1e-12) and co(1000) == pytest.approx(0.0, abs=1e-12)


def test_loss_snr_clip():
    a = torch.tensor([1.0, 2.0, 3.0, 4.0])
    b = torch.tensor([1.0, 2.0, 3.0, 6.0])
    assert float(train.mse_loss(b, a)) == pytest.approx(0.5 * 4 / 4)
    assert train.snr(a, b) == pytest.approx(10 * math.log10(np.var([1, 2, 3, 4]) / 1.0))
    net = inverse.ODPNet(None, depth=3, channels=1, num_filters=2, block_depth=2, alpha_ini=0.5)
    with torch.no_grad():
        net.blocks[1].alpha.fill_(-1.0)
    train.clip_positive(net, minval=1e-3)
    assert [float(b.alpha.detach()) for b in net.blocks] == pytest.approx([0.5, 1e-3, 0.125])


class _DenseOp:
    """A small dense operator with the projector interface (project /
    back_project on batched tensors)."""

    def __init__(self, n, m, seed=0):
        g = torch.Generator().manual_seed(seed)
        self.A = torch.rand((m, n * n), generator=g) / n
        self.input_shape, self.output_shape = (n, n), (m,)

    def project(self, v):
        return (v.reshape(v.shape[0], -1) @ self.A.T).reshape((v.shape[0],) + self.output_shape)

    def back_project(self, w):
        return (w.reshape(w.shape[0], -1) @ self.A).reshape((w.shape[0],) + self.input_shape)


def _toy_data(op, count, seed):
    g = torch.Generator().manual_seed(seed)
    x = torch.rand((count,) + op.input_shape, generator=g)
    return {"image": op.project(x)[..., None].numpy(), "label": x[..., None].numpy()}


def test_odp_training_loop_cpu(tmp_path):
    torch.manual_seed(0)
    op = _DenseOp(8, 40)
    net = inverse.ODPNet(op, depth=2, channels=1, num_filters=4, block_depth=2, alpha_ini=0.05,
                         odp_block=inverse.ODPGrDescBlock)
    cfg = {"device": "cpu", "seed": 1, "opt_type": "ADAM", "batch_size": 4, "num_epochs": 6,
           "base_learning_rate": 1e-2, "log_every_steps": 6, "steps_per_checkpoint": 12, "checkpointing": True,
           "workdir": str(tmp_path), "post_lst": [lambda m: train.clip_positive(m, minval=1e-3)]}
    tr = train.BasicTrainer(cfg, net, _toy_data(op, 16, 2), _toy_data(op, 8, 3))
    assert tr.steps_per_epoch == 4 and tr.num_steps == 24
    state, stats = tr.train()
    assert [r["Epoch"] for r in stats] == [1, 2, 4, 5]
    # training loss falls; eval runs with the batch-norm running statistics,
    # which move slowly (momentum 0.01, the reference's 0.99) and are only
    # checked to be finite here
    assert stats[-1]["Train_Loss"] < 0.5 * stats[0]["Train_Loss"]
    assert all(np.isfinite(r["Eval_Loss"]) and np.isfinite(r["Eval_SNR"]) for r in stats)
    assert all(float(b.alpha) >= 1e-3 for b in net.blocks)
    assert sorted(p.name for p in tmp_path.iterdir()) == ["checkpoint_12.pt", "checkpoint_24.pt"]
    # a new trainer on the same workdir resumes at the last checkpoint: nothing left to run
    net2 = inverse.ODPNet(op, depth=2, channels=1, num_filters=4, block_depth=2, alpha_ini=0.05,
                          odp_block=inverse.ODPGrDescBlock)
    tr2 = train.BasicTrainer(cfg, net2, _toy_data(op, 16, 2), _toy_data(op, 8, 3))
    assert tr2.step == 24
    tr2.train()
    for a, b in zip(net.state_dict().values(), net2.state_dict().values()):
        assert torch.equal(a, b)


class _CircConvOp:
    """Circular convolution with a small blur kernel through the real DFT,
    with the projector interface (project / back_project on batched
    tensors)."""

    def __init__(self, n, seed=0):
        g = torch.Generator().manual_seed(seed)
        k = torch.zeros((n, n))
        k[:3, :3] = torch.rand((3, 3), generator=g)
        k /= k.sum()
        self.kf = torch.fft.rfft2(k)
        self.input_shape = self.output_shape = (n, n)

    def project(self, v):
        return torch.fft.irfft2(torch.fft.rfft2(v) * self.kf, s=self.input_shape)

    def back_project(self, w):
        return torch.fft.irfft2(torch.fft.rfft2(w) * self.kf.conj(), s=self.input_shape)


def test_odp_deconvolution_block():
    """ODPProxDcnvBlock (scico/flax/inverse.py:228-313): ||A|| by power
    iteration equals the largest |K(f)| of the circular convolution, and the
    block's output is (alpha A^T y + ResNet(x)) (alpha ||A||^2 + 1) through the
    DFT round trip."""
    torch.manual_seed(0)
    op = _CircConvOp(16)
    blk = inverse.ODPProxDcnvBlock(op, depth=2, channels=1, num_filters=4, alpha_ini=0.7)
    assert blk.operator_norm == pytest.approx(float(op.kf.abs().max()), rel=1e-4)
    x = torch.rand((3, 16, 16))
    y = op.project(torch.rand((3, 16, 16)))
    out = blk(x, y)
    a = 0.7
    ref = (a * op.back_project(y) + blk.resnet(x.unsqueeze(1)).squeeze(1)) * (a * blk.operator_norm ** 2 + 1)
    assert float((out - ref).norm() / ref.norm()) <= 1e-5
    g = torch.autograd.grad(out.sum(), [blk.alpha])[0]
    assert torch.isfinite(g).all()


def test_odp_deconvolution_training_cpu():
    torch.manual_seed(0)
    op = _CircConvOp(8)
    net = inverse.ODPNet(op, depth=2, channels=1, num_filters=4, block_depth=2, alpha_ini=0.05,
                         odp_block=inverse.ODPProxDcnvBlock)
    cfg = {"device": "cpu", "seed": 1, "opt_type": "ADAM", "batch_size": 4, "num_epochs": 6,
           "base_learning_rate": 1e-2, "log_every_steps": 6, "checkpointing": False}
    tr = train.BasicTrainer(cfg, net, _toy_data(op, 16, 2), _toy_data(op, 8, 3))
    state, stats = tr.train()
    assert stats[-1]["Train_Loss"] < stats[0]["Train_Loss"]
