"""GPU training of the subtree-surrogate GRU with the library's own kernels.

The network (hidden 64, inputs 4, BF16 recurrent weights, FP32 accumulation on
the tensor cores) and its flat parameter layout are those of the C ABI
(``bc_gru_*``).  :class:`GRUTrainer` keeps the sequences, the FP32 master
weights, the Adam moments and the per-window activations in device memory
(PyTorch tensors, used as plain allocations) and runs truncated BPTT: each
window of ``window`` steps of a batch of ``batch`` sequences is one forward
kernel, one backward kernel (all weight gradients accumulated in the same
pass) and one Adam kernel; the hidden state is carried across the windows of a
sequence, the gradient is not.  No autograd and no PyTorch kernels are used on
this path.
"""

from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import _abi

__all__ = ["H", "X", "NPARAM", "init_params", "GRUTrainer", "TrainLog"]

H = _abi.BC_GRU_HIDDEN
X = _abi.BC_GRU_INPUTS
G3 = 3 * H
NPARAM = G3 * H + G3 * X + 2 * G3 + H + 1


def init_params(seed: int = 0, scale: float = 1.0) -> np.ndarray:
    """Uniform(-scale/sqrt(H), scale/sqrt(H)) weights and biases, output bias 0 (float32)."""
    rng = np.random.default_rng(seed)
    k = scale / np.sqrt(H)
    theta = rng.uniform(-k, k, size=NPARAM).astype(np.float32)
    theta[-1] = 0.0
    return theta


def _ptr(t) -> C.c_void_p:
    return C.c_void_p(int(t.data_ptr())) if t is not None else C.c_void_p(0)


@dataclass
class TrainLog:
    updates: int = 0
    epochs: int = 0
    seconds: float = 0.0
    loss: list = field(default_factory=list)       # mean window loss per epoch
    val_loss: list = field(default_factory=list)   # held-out mean squared error per epoch


class GRUTrainer:
    """Truncated-BPTT Adam training of the GRU on sequences ``x [n, T, 4]``, ``y [n, T]``."""

    def __init__(self, x: np.ndarray, y: np.ndarray, theta0: np.ndarray | None = None, *, batch: int = 512,
                 window: int = 400, lr: float = 1e-3, betas=(0.9, 0.999), eps: float = 1e-8, clip: float = 1.0,
                 device: int = 0, seed: int = 0):
        import torch

        if x.ndim != 3 or x.shape[2] != X or y.shape != x.shape[:2]:
            raise ValueError(f"x must be [n, T, {X}] and y [n, T].")
        self._lib = _abi.lib()
        if int(self._lib.bc_gru_nparam()) != NPARAM:
            raise RuntimeError("GRU parameter layout differs between Python and the native library.")
        self.torch = torch
        self.dev = torch.device("cuda", device)
        self.n_seq, self.t_total = int(x.shape[0]), int(x.shape[1])
        self.batch = int(min(batch, self.n_seq))
        self.window = int(min(window, self.t_total))
        self.lr, self.betas, self.eps, self.clip = float(lr), betas, float(eps), float(clip)
        self.rng = np.random.default_rng(seed)
        f32 = torch.float32
        self.x = torch.as_tensor(np.ascontiguousarray(x, np.float32)).to(self.dev)
        self.y = torch.as_tensor(np.ascontiguousarray(y, np.float32)).to(self.dev)
        theta = init_params(seed) if theta0 is None else np.asarray(theta0, np.float32)
        self.params = torch.as_tensor(theta.copy()).to(self.dev)
        self.grads = torch.zeros(NPARAM, dtype=f32, device=self.dev)
        # per-CTA gradient rows of the backward, summed in a fixed order
        self.work = torch.zeros(int(self._lib.bc_gru_backward_workspace(self.batch)), dtype=f32, device=self.dev)
        self.m = torch.zeros(NPARAM, dtype=f32, device=self.dev)
        self.v = torch.zeros(NPARAM, dtype=f32, device=self.dev)
        self.wext = torch.zeros(4 * H * (H + 16) // 2, dtype=torch.int32, device=self.dev)
        self.wht = torch.zeros(G3 * H // 2, dtype=torch.int32, device=self.dev)
        self.acts = torch.zeros((5, self.batch, self.window, H), dtype=f32, device=self.dev)
        self.yout = torch.zeros((self.batch, self.window), dtype=f32, device=self.dev)
        self.h = torch.zeros((self.batch, H), dtype=f32, device=self.dev)
        self.loss = torch.zeros(1, dtype=torch.float64, device=self.dev)
        self.sq = torch.zeros(1, dtype=f32, device=self.dev)
        self.seq = torch.zeros(self.batch, dtype=torch.int32, device=self.dev)
        self.step_count = 0
        self.log = TrainLog()
        self._pack()

    # ------------------------------------------------------------------ kernels
    def _stream(self):
        return C.c_void_p(int(self.torch.cuda.current_stream(self.dev).cuda_stream))

    def _pack(self) -> None:
        _abi.check(self._lib.bc_gru_pack(_ptr(self.params), _ptr(self.wext), _ptr(self.wht), self._stream()))

    def _set_batch(self, seq_ids: np.ndarray) -> int:
        b = int(seq_ids.size)
        self.seq[:b].copy_(self.torch.as_tensor(seq_ids.astype(np.int32)))
        return b

    def forward_window(self, b: int, t0: int, T: int, store: bool = True) -> None:
        _abi.check(self._lib.bc_gru_forward(
            _ptr(self.params), _ptr(self.wext), _ptr(self.x), _ptr(self.y), self.t_total, _ptr(self.seq), b, t0, T,
            _ptr(self.h), _ptr(self.acts) if store else None, _ptr(self.yout), _ptr(self.loss), self._stream()))

    def backward_window(self, b: int, t0: int, T: int) -> None:
        _abi.check(self._lib.bc_gru_backward(
            _ptr(self.params), _ptr(self.wht), _ptr(self.x), _ptr(self.y), self.t_total, _ptr(self.seq), b, t0, T,
            _ptr(self.acts), _ptr(self.yout), C.c_float(2.0 / (b * T)), _ptr(self.grads), _ptr(self.work),
            self._stream()))

    def adam_step(self) -> None:
        self.step_count += 1
        scale = 1.0
        if self.clip > 0:
            _abi.check(self._lib.bc_gru_grad_sqnorm(_ptr(self.grads), _ptr(self.sq), self._stream()))
            norm = float(self.sq.item()) ** 0.5
            scale = min(1.0, self.clip / norm) if norm > 0 else 1.0
        b1, b2 = self.betas
        _abi.check(self._lib.bc_gru_adam(_ptr(self.params), _ptr(self.grads), _ptr(self.m), _ptr(self.v),
                                         self.step_count, C.c_float(self.lr), C.c_float(b1), C.c_float(b2),
                                         C.c_float(self.eps), C.c_float(scale), self._stream()))
        self._pack()

    # ------------------------------------------------------------------ API
    def gradient(self, seq_ids, t0: int, T: int, h0: np.ndarray | None = None) -> tuple[float, np.ndarray, np.ndarray]:
        """(mean loss, gradient, outputs) of one window (the state is not carried)."""
        seq_ids = np.asarray(seq_ids)
        b = self._set_batch(seq_ids)
        if T > self.window or b > self.batch:
            raise ValueError("window or batch larger than the trainer's buffers.")
        self.h.zero_()
        if h0 is not None:
            self.h[:b].copy_(self.torch.as_tensor(np.asarray(h0, np.float32)))
        self.loss.zero_()
        self.grads.zero_()
        self.forward_window(b, t0, T)
        self.backward_window(b, t0, T)
        self.torch.cuda.synchronize(self.dev)
        yout = self.yout.view(-1)[:b * T].reshape(b, T).cpu().numpy().astype(np.float64)
        return float(self.loss.item()) / (b * T), self.grads.cpu().numpy().astype(np.float64), yout

    def train(self, epochs: int = 10, time_budget_s: float | None = None, val: tuple | None = None,
              log_every: int = 1, lr_final: float | None = None) -> TrainLog:
        """Epochs over all sequences (random batches, windows in time order).  With
        ``lr_final`` the learning rate follows a cosine from ``lr`` to ``lr_final``."""
        t_start = time.perf_counter()
        lr0 = self.lr
        for ep in range(epochs):
            if lr_final is not None:
                self.lr = lr_final + 0.5 * (lr0 - lr_final) * (1.0 + math.cos(math.pi * ep / max(epochs, 1)))
            order = self.rng.permutation(self.n_seq)
            ep_loss, n_win = 0.0, 0
            for s0 in range(0, self.n_seq, self.batch):
                ids = order[s0:s0 + self.batch]
                b = self._set_batch(ids)
                self.h.zero_()
                for t0 in range(0, self.t_total, self.window):
                    T = min(self.window, self.t_total - t0)
                    self.loss.zero_()
                    self.forward_window(b, t0, T)
                    self.backward_window(b, t0, T)
                    self.adam_step()
                    ep_loss += float(self.loss.item()) / (b * T)
                    n_win += 1
                    self.log.updates += 1
                if time_budget_s is not None and time.perf_counter() - t_start > time_budget_s:
                    break
            self.log.epochs += 1
            self.log.loss.append(ep_loss / max(n_win, 1))
            if val is not None and (ep % log_every == 0 or ep == epochs - 1):
                self.log.val_loss.append(self.evaluate(*val))
            if time_budget_s is not None and time.perf_counter() - t_start > time_budget_s:
                break
        self.torch.cuda.synchronize(self.dev)
        self.lr = lr0
        self.log.seconds += time.perf_counter() - t_start
        return self.log

    def predict(self, x: np.ndarray) -> np.ndarray:
        """Outputs of the current network on sequences ``x [n, T, 4]`` from h = 0."""
        torch = self.torch
        n, T = int(x.shape[0]), int(x.shape[1])
        xd = torch.as_tensor(np.ascontiguousarray(x, np.float32)).to(self.dev)
        out = np.zeros((n, T), np.float64)
        yout = torch.zeros((self.batch, T), dtype=torch.float32, device=self.dev)
        h = torch.zeros((self.batch, H), dtype=torch.float32, device=self.dev)
        for s0 in range(0, n, self.batch):
            ids = np.arange(s0, min(s0 + self.batch, n))
            b = self._set_batch(ids)
            h.zero_()
            _abi.check(self._lib.bc_gru_forward(
                _ptr(self.params), _ptr(self.wext), _ptr(xd), None, T, _ptr(self.seq), b, 0, T, _ptr(h), None,
                _ptr(yout), None, self._stream()))
            torch.cuda.synchronize(self.dev)
            out[s0:s0 + b] = yout[:b].cpu().numpy()
        return out

    def evaluate(self, x: np.ndarray, y: np.ndarray) -> float:
        return float(np.mean((self.predict(x) - y) ** 2))

    def theta(self) -> np.ndarray:
        self.torch.cuda.synchronize(self.dev)
        return self.params.cpu().numpy().copy()
