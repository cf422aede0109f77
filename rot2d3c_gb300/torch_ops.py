"""PyTorch binding of the learned closure over the C-ABI.

``rot2d3c::cnn_forward`` is a ``torch.library`` custom operator whose
forward calls ``r2d3c_cnn_forward`` and whose backward calls
``r2d3c_cnn_backward`` (the network's own BF16 tensor-core kernels), so the
closure network can sit inside any PyTorch graph: losses, optimisers and
schedulers written in PyTorch train it through autograd.  The parameters are
a torch tensor (FP32, the C-ABI's parameter layout); when it has changed
since the last call (an optimiser step) it is copied into the network before
the call.  The solver's own captured LES step (r2d3c_closure_advance) uses
the same network and parameters.

No counterpart in the reference program (it has no learned closure).
"""
from __future__ import annotations

import itertools

import torch

from .closure import CNN

_NETS: dict = {}
_IDS = itertools.count(1)
_PUSHED: dict = {}  # net id -> (data_ptr, version) of the parameters last copied in


def _push(net_id: int, params: torch.Tensor) -> CNN:
    net = _NETS[net_id]
    key = (params.data_ptr(), params._version)
    if _PUSHED.get(net_id) != key:
        net.set_params(params.detach().float().cpu().numpy())
        _PUSHED[net_id] = key
    return net


@torch.library.custom_op("rot2d3c::cnn_forward", mutates_args=())
def cnn_forward(x: torch.Tensor, params: torch.Tensor, net_id: int) -> torch.Tensor:
    """Network output [B, H, W, 2] for inputs x [B, H, W, 8] (FP32, CUDA)."""
    net = _push(net_id, params)
    x = x.contiguous()
    out = torch.empty(x.shape[:-1] + (2,), dtype=torch.float32, device=x.device)
    net.forward(x, x.shape[0], out)
    return out


@cnn_forward.register_fake
def _(x, params, net_id):
    return x.new_empty(x.shape[:-1] + (2,))


@torch.library.custom_op("rot2d3c::cnn_vjp", mutates_args=())
def cnn_vjp(x: torch.Tensor, params: torch.Tensor, gout: torch.Tensor,
            net_id: int) -> tuple[torch.Tensor, torch.Tensor]:
    """(dL/dx, dL/dparams) for dL/d(output) = gout."""
    net = _push(net_id, params)
    x = x.contiguous()
    gx = torch.empty_like(x)
    g = net.backward(x, gout.contiguous().float(), x.shape[0], gx)
    return gx, torch.from_numpy(g).to(params.device)


@cnn_vjp.register_fake
def _(x, params, gout, net_id):
    return x.new_empty(x.shape), params.new_empty(params.shape)


def _setup_context(ctx, inputs, output):
    x, params, net_id = inputs
    ctx.save_for_backward(x, params)
    ctx.net_id = net_id


def _backward(ctx, gout):
    x, params = ctx.saved_tensors
    gx, gp = cnn_vjp(x, params, gout, ctx.net_id)
    return gx, gp, None


cnn_forward.register_autograd(_backward, setup_context=_setup_context)


class ClosureNet(torch.nn.Module):
    """The closure CNN as a torch module: ``params`` is its parameter
    vector (torch.nn.Parameter on the GPU), ``net`` the C-ABI network."""

    def __init__(self, H: int, W: int, max_batch: int, seed: int = 0):
        super().__init__()
        self.net = CNN(H, W, max_batch, seed)
        self.net_id = next(_IDS)
        _NETS[self.net_id] = self.net
        self.params = torch.nn.Parameter(torch.from_numpy(self.net.get_params()).cuda())

    def set_normalization(self, in_mean, in_std, out_mean, out_std) -> None:
        self.net.set_normalization(in_mean, in_std, out_mean, out_std)

    def forward(self, x: torch.Tensor) -> torch.Tensor:
        return cnn_forward(x, self.params, self.net_id)
