"""The per-point MLP on the BF16 tensor cores (tcgen05), as a torch-facing
object over ``ice3gb_mlp_*`` of include/ice3gb.h.

``n_in -> n_hidden (GELU) x n_hidden_layers -> n_out``: BF16 weights and
activations, FP32 accumulation in TMEM, FP32 master weights and Adam; the
forward and the hand-written backward pass run in the library's own GEMM
kernel (no cuBLAS).  Inputs and outputs are FP32 CUDA tensors.

The loss is the surrogate head's: per rate r, output 2r is the logit of
"the rate is nonzero" (binary cross-entropy against target 2r in {0, 1}) and
output 2r + 1 the transformed rate (squared error against target 2r + 1,
counted only where the rate is nonzero); the mean over the batch.  Targets
are [n][16] (columns past n_out are ignored).
"""
from __future__ import annotations

import ctypes
from typing import List, Tuple

import numpy as np
import torch

from . import _abi


def _ptr(t: torch.Tensor) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr())


def _stream() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class Mlp:
    def __init__(self, n_in: int = 16, n_hidden: int = 256, n_hidden_layers: int = 3, n_out: int = 10,
                 seed: int = 0):
        self.lib = _abi.load()
        self.shape = (n_in, n_hidden, n_hidden_layers, n_out)
        s = _abi.MlpShape(n_in, n_hidden, n_hidden_layers, n_out)
        h = ctypes.c_void_p()
        _abi.check(self.lib.ice3gb_mlp_create(ctypes.byref(s), ctypes.c_uint64(seed), ctypes.byref(h)), None,
                   "ice3gb_mlp_create")
        self.h = h
        self.n_params = int(self.lib.ice3gb_mlp_param_count(h))

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value:
            try:
                self.lib.ice3gb_mlp_destroy(h)
            except Exception:
                pass
            self.h = None

    # ---- parameters -----------------------------------------------------
    def layout(self) -> List[Tuple[int, int, int, int]]:
        """(W offset, b offset, out, in) per weight layer of the flat vector."""
        n_in, n_hid, nh, n_out = self.shape
        out, off = [], 0
        for l in range(nh + 1):
            din = n_in if l == 0 else n_hid
            dout = n_out if l == nh else n_hid
            out.append((off, off + din * dout, dout, din))
            off += din * dout + dout
        return out

    def get_params(self) -> np.ndarray:
        p = np.empty(self.n_params, dtype=np.float32)
        _abi.check(self.lib.ice3gb_mlp_get_params(self.h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float))), None,
                   "ice3gb_mlp_get_params")
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters, got {p.size}")
        _abi.check(self.lib.ice3gb_mlp_set_params(self.h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float))), None,
                   "ice3gb_mlp_set_params")

    # ---- compute ----------------------------------------------------------
    def _check_x(self, x: torch.Tensor) -> torch.Tensor:
        if not (x.is_cuda and x.dtype == torch.float32 and x.dim() == 2 and x.shape[1] == self.shape[0]):
            raise ValueError(f"x must be a float32 CUDA tensor [n, {self.shape[0]}]")
        return x.contiguous()

    def _check_t(self, t: torch.Tensor, n: int) -> torch.Tensor:
        if not (t.is_cuda and t.dtype == torch.float32 and tuple(t.shape) == (n, 16)):
            raise ValueError("targets must be a float32 CUDA tensor [n, 16]")
        return t.contiguous()

    def forward(self, x: torch.Tensor) -> torch.Tensor:
        x = self._check_x(x)
        y = torch.empty((x.shape[0], self.shape[3]), dtype=torch.float32, device=x.device)
        _abi.check(self.lib.ice3gb_mlp_forward(self.h, int(x.shape[0]), _ptr(x), _ptr(y), _stream()), None,
                   "ice3gb_mlp_forward")
        return y

    __call__ = forward

    def forward_layered(self, x: torch.Tensor) -> torch.Tensor:
        """The same forward with one GEMM launch per layer (the training path)."""
        x = self._check_x(x)
        y = torch.empty((x.shape[0], self.shape[3]), dtype=torch.float32, device=x.device)
        _abi.check(self.lib.ice3gb_mlp_forward_layered(self.h, int(x.shape[0]), _ptr(x), _ptr(y), _stream()), None,
                   "ice3gb_mlp_forward_layered")
        return y

    def loss_grad(self, x: torch.Tensor, targets: torch.Tensor) -> Tuple[float, torch.Tensor]:
        x = self._check_x(x)
        t = self._check_t(targets, x.shape[0])
        g = torch.empty(self.n_params, dtype=torch.float32, device=x.device)
        loss = torch.empty(1, dtype=torch.float32, device=x.device)
        _abi.check(self.lib.ice3gb_mlp_loss_grad(self.h, int(x.shape[0]), _ptr(x), _ptr(t), _ptr(g), _ptr(loss),
                                                 _stream()), None, "ice3gb_mlp_loss_grad")
        return float(loss.item()), g

    def train_step(self, x: torch.Tensor, targets: torch.Tensor, lr: float, loss: torch.Tensor = None) -> None:
        """One Adam step on one batch; the loss goes to ``loss`` (a float32
        CUDA tensor of one element) when given, without a synchronisation."""
        x = self._check_x(x)
        t = self._check_t(targets, x.shape[0])
        lp = _ptr(loss) if loss is not None else ctypes.c_void_p(0)
        _abi.check(self.lib.ice3gb_mlp_train_step(self.h, int(x.shape[0]), _ptr(x), _ptr(t), ctypes.c_float(lr), lp,
                                                  _stream()), None, "ice3gb_mlp_train_step")

    def check(self) -> None:
        """Raise if a tensor-core kernel of this MLP timed out on its barrier."""
        _abi.check(self.lib.ice3gb_mlp_error(self.h), None, "tensor-core MLP")


def tc_gemm_bf16(a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """C = A B^T in FP32 on the tensor cores for BF16 CUDA tensors A [M, K]
    and B [N, K] of any strides (N <= 256)."""
    if a.dtype != torch.bfloat16 or b.dtype != torch.bfloat16 or not (a.is_cuda and b.is_cuda):
        raise ValueError("bf16 CUDA tensors expected")
    M, K = a.shape
    N, K2 = b.shape
    if K2 != K:
        raise ValueError("inner dimensions differ")
    c = torch.empty((M, N), dtype=torch.float32, device=a.device)
    err = torch.zeros(1, dtype=torch.int32, device=a.device)
    lib = _abi.load()
    _abi.check(lib.ice3gb_tc_gemm_bf16(M, N, K, _ptr(a), a.stride(0), a.stride(1), _ptr(b), b.stride(0),
                                       b.stride(1), _ptr(c), c.stride(0), _ptr(err), _stream()), None,
               "ice3gb_tc_gemm_bf16")
    if int(err.item()) != 0:
        raise _abi.Ice3gbError("tc_gemm_bf16: tensor-core barrier timed out")
    return c


def main(argv=None) -> int:
    """Time the surrogate-shaped network's inference on random rows:
    python -m ice3gb.mlp --rows 8388608 --reps 5 [--layered]"""
    import argparse
    import json
    ap = argparse.ArgumentParser()
    ap.add_argument("--rows", type=int, default=1 << 23)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--layered", action="store_true", help="one GEMM launch per layer instead of the fused kernel")
    a = ap.parse_args(argv)
    net = Mlp(16, 256, 3, 10, seed=0)
    gen = torch.Generator(device="cuda").manual_seed(0)
    x = torch.randn((a.rows, 16), generator=gen, device="cuda")
    fwd = net.forward_layered if a.layered else net.forward
    fwd(x)
    torch.cuda.synchronize()
    times = []
    for _ in range(a.reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fwd(x)
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    net.check()
    ms = min(times)
    flop = a.rows * 2 * (16 * 256 + 2 * 256 * 256 + 256 * 10)
    print(json.dumps({"rows": a.rows, "path": "layered" if a.layered else "fused", "ms_best": ms,
                      "rows_per_s": a.rows / ms * 1e3, "tflops": flop / ms / 1e9}))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
