"""Training driver for the unrolled reconstruction networks (MoDLNet, ODPNet)
on the GPU operators: the training workflow of scico.flax.train
(scico/flax/train/trainer.py, steps.py, learning_rate.py, losses.py,
diagnostics.py, traversals.py) restated for torch modules.

Configuration keys follow the reference's ConfigDict
(scico/flax/train/trainer.py:62-300): ``seed``, ``opt_type`` ("SGD",
"ADAM", "ADAMW"), ``momentum``, ``weight_decay``, ``batch_size``,
``num_epochs``, ``base_learning_rate``, ``lr_decay_rate``,
``warmup_epochs``, ``lr_schedule``, ``criterion``, ``steps_per_eval``,
``steps_per_checkpoint``, ``log_every_steps``, ``log``, ``workdir``,
``checkpointing``, ``return_state``, ``post_lst`` (and ``device``, default
the CUDA device; ``cudnn_search``, default True: cuDNN picks convolution
algorithms by measuring them, as XLA autotunes the reference's
convolutions).  Data sets are dicts with
``"image"`` (the network input: projections ``(N, *A.output_shape)``, an
optional trailing channel axis of 1) and ``"label"`` (the images).

One process, one GPU: the reference's data-parallel replication (``pmap``
over devices, cross-replica batch statistics) has nothing to replicate here.
"""

from __future__ import annotations

import math
import os
import time
from typing import Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _device


# ---------------------------------------------------------------------------
# losses and metrics (losses.py:17-28, scico/metric.py:48-62)
# ---------------------------------------------------------------------------


def mse_loss(output: torch.Tensor, labels: torch.Tensor) -> torch.Tensor:
    """Mean of optax's l2 loss, ``0.5 (output - labels)^2``."""
    return 0.5 * torch.mean((output - labels) ** 2)


def snr(reference: torch.Tensor, comparison: torch.Tensor) -> float:
    """10 log10(var(reference) / mse(reference, comparison)) in dB."""
    ref = reference.double()
    mse = torch.mean((ref - comparison.double()) ** 2)
    return float(10.0 * torch.log10(torch.var(ref, unbiased=False) / mse))


def compute_metrics(output: torch.Tensor, labels: torch.Tensor, criterion: Callable = mse_loss) -> Dict[str, float]:
    """Loss and SNR of a batch (diagnostics.py:25-45)."""
    return {"loss": float(criterion(output, labels)), "snr": snr(labels, output)}


# ---------------------------------------------------------------------------
# learning-rate schedules (learning_rate.py): functions of the step count
# ---------------------------------------------------------------------------


def create_cnst_lr_schedule(config) -> Callable[[int], float]:
    """Constant ``base_learning_rate``."""
    lr = float(config["base_learning_rate"])
    return lambda step: lr


def create_exp_lr_schedule(config) -> Callable[[int], float]:
    """``base_learning_rate * lr_decay_rate ** (step / decay_steps)`` with
    decay_steps = num_epochs * steps_per_epoch (optax.exponential_decay)."""
    lr0, rate = float(config["base_learning_rate"]), float(config["lr_decay_rate"])
    decay_steps = max(1, int(config["num_epochs"]) * int(config["steps_per_epoch"]))
    return lambda step: lr0 * rate ** (step / decay_steps)


def create_cosine_lr_schedule(config) -> Callable[[int], float]:
    """Linear warm-up from 0 over ``warmup_epochs``, then cosine decay to 0
    over the remaining epochs (at least one)."""
    lr0 = float(config["base_learning_rate"])
    spe = int(config["steps_per_epoch"])
    warm = int(config.get("warmup_epochs", 0)) * spe
    decay = max(int(config["num_epochs"]) - int(config.get("warmup_epochs", 0)), 1) * spe

    def schedule(step):
        if step < warm:
            return lr0 * step / warm
        t = min(step - warm, decay) / decay
        return lr0 * 0.5 * (1.0 + math.cos(math.pi * t))

    return schedule


# ---------------------------------------------------------------------------
# parameter post-processing (traversals.py:31-60)
# ---------------------------------------------------------------------------


def _selected(model: torch.nn.Module, names: Sequence[str]):
    return [p for n, p in model.named_parameters() if n.split(".")[-1] in names]


def clip_positive(model: torch.nn.Module, names: Sequence[str] = ("alpha",), minval: float = 1e-4) -> None:
    """Clamp the named scalar parameters (``alpha``, ``lmbda``) to at least
    ``minval``."""
    with torch.no_grad():
        for p in _selected(model, names):
            p.clamp_(min=minval)


def clip_range(model: torch.nn.Module, names: Sequence[str] = ("alpha",), minval: float = 1e-4,
               maxval: float = 1.0) -> None:
    """Clamp the named parameters to [minval, maxval]."""
    with torch.no_grad():
        for p in _selected(model, names):
            p.clamp_(min=minval, max=maxval)


# ---------------------------------------------------------------------------
# data
# ---------------------------------------------------------------------------


def _as_tensor(a, dev) -> torch.Tensor:
    t = torch.as_tensor(np.asarray(a) if not isinstance(a, torch.Tensor) else a, dtype=torch.float32)
    if t.ndim >= 3 and t.shape[-1] == 1:  # the reference's NHWC channel axis
        t = t[..., 0]
    return t.to(dev).contiguous()


class _Batches:
    """Shuffled full batches of a data set, reshuffled every epoch
    (input_pipeline.py:38-88); the data stay on the device."""

    def __init__(self, ds, batch_size: int, dev, shuffle: bool, seed: int):
        self.x = _as_tensor(ds["image"], dev)
        self.y = _as_tensor(ds["label"], dev)
        if len(self.x) != len(self.y):
            raise ValueError("image and label counts differ")
        self.n, self.bs, self.shuffle = len(self.x), batch_size, shuffle
        self.gen = torch.Generator().manual_seed(seed)
        self._reset()

    def _reset(self):
        self.perm = torch.randperm(self.n, generator=self.gen) if self.shuffle else torch.arange(self.n)
        self.pos = 0

    def next(self) -> Tuple[torch.Tensor, torch.Tensor]:
        if self.pos + self.bs > self.n:
            self._reset()
        idx = self.perm[self.pos:self.pos + self.bs].to(self.x.device)
        self.pos += self.bs
        return self.x[idx], self.y[idx]


# ---------------------------------------------------------------------------
# trainer (trainer.py:56-540)
# ---------------------------------------------------------------------------


class BasicTrainer:
    """Training and evaluation loop of a reconstruction network.

    ``train()`` runs ``num_epochs * (len(train) // batch_size)`` optimizer
    steps on shuffled batches, applies every ``post_lst`` function to the
    model after each step, evaluates loss and SNR on ``steps_per_eval``
    test batches every ``log_every_steps`` steps, and saves a checkpoint
    every ``steps_per_checkpoint`` steps and at the end when
    ``checkpointing`` is set (resuming from the latest one in ``workdir``).
    Returns the model's state dict (or the model itself with
    ``return_state``) and the list of logged statistics.
    """

    STAT_FIELDS = ("Epoch", "Time", "Train_LR", "Train_Loss", "Train_SNR", "Eval_Loss", "Eval_SNR")

    def __init__(self, config: dict, model: torch.nn.Module, train_ds: dict, test_ds: dict):
        self.config = dict(config)
        # the CT operators run on the CUDA device; a network over other
        # (dense, CPU) operators may name its device
        self.dev = torch.device(config["device"]) if "device" in config else _device.require_cuda()
        self.model = model.to(self.dev)
        if self.dev.type == "cuda":
            torch.backends.cudnn.benchmark = bool(config.get("cudnn_search", True))
        seed = int(config.get("seed", 0))
        torch.manual_seed(seed)
        bs = int(config.get("batch_size", 2))
        self.num_epochs = int(config.get("num_epochs", 10))
        n_train = len(train_ds["image"])
        n_test = len(test_ds["image"])
        self.steps_per_epoch = n_train // bs
        if self.steps_per_epoch < 1:
            raise ValueError(f"batch_size {bs} is larger than the training set ({n_train})")
        self.config["steps_per_epoch"] = self.steps_per_epoch
        self.num_steps = self.steps_per_epoch * self.num_epochs
        self.steps_per_eval = int(config.get("steps_per_eval", max(1, n_test // bs)))
        self.steps_per_checkpoint = int(config.get("steps_per_checkpoint", self.steps_per_epoch * 10))
        self.log_every_steps = int(config.get("log_every_steps", self.steps_per_epoch * 20))
        self.logflag = bool(config.get("log", False))
        self.workdir = config.get("workdir", os.path.join(os.path.expanduser("~"), ".cache", "scico_gb300"))
        self.checkpointing = bool(config.get("checkpointing", False))
        self.return_state = bool(config.get("return_state", False))
        self.lr_schedule = config.get("lr_schedule", create_cnst_lr_schedule)(self.config)
        self.criterion = config.get("criterion", mse_loss)
        self.post_lst: List[Callable] = list(config.get("post_lst", []))
        self.train_it = _Batches(train_ds, bs, self.dev, True, seed)
        self.eval_it = _Batches(test_ds, min(bs, n_test), self.dev, False, seed)
        self.optimizer = self._optimizer()
        self.step = 0
        self.stats: List[dict] = []
        if self.checkpointing:
            self._restore()

    def _optimizer(self) -> torch.optim.Optimizer:
        opt = self.config.get("opt_type", "ADAM")
        lr = self.lr_schedule(0)
        params = self.model.parameters()
        if opt == "SGD":
            if "momentum" in self.config:
                return torch.optim.SGD(params, lr=lr, momentum=float(self.config["momentum"]), nesterov=True)
            return torch.optim.SGD(params, lr=lr)
        if opt == "ADAM":
            return torch.optim.Adam(params, lr=lr)
        if opt == "ADAMW":
            return torch.optim.AdamW(params, lr=lr, weight_decay=float(self.config.get("weight_decay", 1e-4)))
        raise NotImplementedError(f"Optimizer specified {opt} has not been included in scico_gb300")

    def _ckpt_path(self, step: int) -> str:
        return os.path.join(self.workdir, f"checkpoint_{step}.pt")

    def _restore(self):
        if not os.path.isdir(self.workdir):
            return
        steps = [int(f[11:-3]) for f in os.listdir(self.workdir) if f.startswith("checkpoint_") and f.endswith(".pt")]
        if not steps:
            return
        ck = torch.load(self._ckpt_path(max(steps)), map_location=self.dev)
        self.model.load_state_dict(ck["model"])
        self.optimizer.load_state_dict(ck["optimizer"])
        self.step = int(ck["step"])

    def checkpoint(self):
        if not self.checkpointing:
            return
        os.makedirs(self.workdir, exist_ok=True)
        torch.save({"model": self.model.state_dict(), "optimizer": self.optimizer.state_dict(), "step": self.step},
                   self._ckpt_path(self.step))

    def train_step(self, x: torch.Tensor, y: torch.Tensor) -> Dict[str, float]:
        """One optimizer step on a batch (steps.py:26-90), then post_lst."""
        lr = self.lr_schedule(self.step)
        for g in self.optimizer.param_groups:
            g["lr"] = lr
        self.model.train()
        self.optimizer.zero_grad(set_to_none=True)
        out = self.model(x)
        loss = self.criterion(out, y)
        loss.backward()
        self.optimizer.step()
        for fn in self.post_lst:
            fn(self.model)
        self.step += 1
        m = compute_metrics(out.detach(), y, self.criterion)
        m["learning_rate"] = lr
        return m

    @torch.no_grad()
    def evaluate(self) -> Dict[str, float]:
        """Mean loss and SNR over ``steps_per_eval`` test batches (eval mode:
        batch normalization uses its running statistics)."""
        self.model.eval()
        ms = []
        for _ in range(self.steps_per_eval):
            x, y = self.eval_it.next()
            ms.append(compute_metrics(self.model(x), y, self.criterion))
        return {k: float(np.mean([m[k] for m in ms])) for k in ms[0]}

    def train(self):
        t0 = time.time()
        window: List[dict] = []
        while self.step < self.num_steps:
            x, y = self.train_it.next()
            window.append(self.train_step(x, y))
            if self.step % self.log_every_steps == 0 or self.step == self.num_steps:
                self._log(window, t0)
                window = []
            if self.step % self.steps_per_checkpoint == 0:
                self.checkpoint()
        self.checkpoint()
        self.train_time = time.time() - t0
        state = self.model if self.return_state else self.model.state_dict()
        return state, self.stats

    def _log(self, window: List[dict], t0: float):
        if not window:
            return
        ev = self.evaluate()
        rec = {"Epoch": (self.step - 1) // self.steps_per_epoch, "Time": time.time() - t0,
               "Train_LR": window[-1]["learning_rate"], "Train_Loss": float(np.mean([m["loss"] for m in window])),
               "Train_SNR": float(np.mean([m["snr"] for m in window])), "Eval_Loss": ev["loss"],
               "Eval_SNR": ev["snr"]}
        self.stats.append(rec)
        if self.logflag:
            print("  ".join(f"{k} {v:.6g}" for k, v in rec.items()), flush=True)

