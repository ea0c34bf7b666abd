"""PyTorch binding: trace sampling on CUDA tensors, and a torch.autograd
binding of the radical-pair yields.

`yield_objective(params, ...)` returns wS*Phi_S + wT*Phi_T of the stepwise
trace-sampling propagation as a 0-d float64 tensor whose backward is the
adjoint gradient of spc_yield_gradient (no finite differences, no tape). The
parameter vector uses the C layout of spc_yield_gradient:

    [Bx, By, Bz, J, D (9, column-major), kS, kT, A (9 per nucleus, column-major)]

in internal units (mT; kS, kT in 1/us divided by gamma_e). `pack_params` and
`unpack_params` convert to and from a SysParam and a field vector.
"""
from __future__ import annotations

import copy

import numpy as np
import torch

from .dynamics import TraceSampler
from .spinsys import SysParam


def pack_params(sys: SysParam, B) -> torch.Tensor:
    Bv = np.array([0.0, 0.0, float(B)]) if np.isscalar(B) else np.asarray(B, np.float64).reshape(3)
    A = [np.asarray(a, np.float64).reshape(3, 3).T.reshape(9) for a in list(sys.e1.A) + list(sys.e2.A)]
    v = np.concatenate([Bv, [sys.J], np.asarray(sys.D, np.float64).reshape(3, 3).T.reshape(9),
                        [sys.kS, sys.kT]] + A)
    return torch.from_numpy(v)


def unpack_params(template: SysParam, v) -> tuple:
    v = np.asarray(v, np.float64)
    n1 = len(template.e1.g_I)
    nn = n1 + len(template.e2.g_I)
    if v.size != 15 + 9 * nn:
        raise ValueError(f"parameter vector has {v.size} entries, the system needs {15 + 9 * nn}")
    s = copy.deepcopy(template)
    A = [v[15 + 9 * j:24 + 9 * j].reshape(3, 3).T.copy() for j in range(nn)]
    s.e1.A, s.e2.A = A[:n1], A[n1:]
    s.J = float(v[3])
    s.D = v[4:13].reshape(3, 3).T.copy()
    s.kS, s.kT = float(v[13]), float(v[14])
    return s, v[0:3].copy()


class _Yield(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, sampler, template, zkets, dt, t_end, m, n_quad, checkpoint_every, wS, wT):
        s, B = unpack_params(template, params.detach().cpu().numpy())
        if ctx.needs_input_grad[0]:
            g = sampler.yield_gradient(s, B, zkets, dt, t_end, m, n_quad=n_quad,
                                       checkpoint_every=checkpoint_every, wS=wS, wT=wT)
            ctx.save_for_backward(torch.from_numpy(g.raw).to(params))
            val = wS * g.Phi_S + wT * g.Phi_T
        else:
            PhiS, PhiT = sampler.stepwise_yields(s, B, zkets, dt, t_end, m)
            val = wS * PhiS + wT * PhiT
        return params.new_tensor(val)

    @staticmethod
    def backward(ctx, grad_out):
        (g,) = ctx.saved_tensors
        return (grad_out * g,) + (None,) * 10


def yield_objective(params: torch.Tensor, sampler: TraceSampler, template: SysParam, zkets,
                    dt: float, t_end: float, m: int, n_quad: int = 0, checkpoint_every: int = 0,
                    wS: float = 1.0, wT: float = 0.0) -> torch.Tensor:
    """wS*Phi_S + wT*Phi_T at `params` (float64, C layout); differentiable
    with respect to params through the adjoint sweep."""
    if params.dtype != torch.float64:
        raise TypeError("params must be float64")
    return _Yield.apply(params, sampler, template, zkets, dt, t_end, m, n_quad, checkpoint_every, wS, wT)


def _device_samples(zkets: torch.Tensor) -> torch.Tensor:
    if not (isinstance(zkets, torch.Tensor) and zkets.is_cuda and zkets.dtype == torch.complex128):
        raise TypeError("zkets must be a CUDA complex128 tensor (samples x Z)")
    return zkets.contiguous()


_SIDE = {}


def _ordered_call(sampler: TraceSampler, device, tensors, fn) -> None:
    """Run fn (library launches) on a torch stream of this module that waits
    for the caller's current stream first and that the caller's stream waits
    for afterwards, so the call is ordered like a torch op on any stream
    (including the legacy default stream, which the library's own
    non-blocking stream would not be ordered against)."""
    cur = torch.cuda.current_stream(device)
    side = _SIDE.get(device)
    if side is None:
        side = _SIDE[device] = torch.cuda.Stream(device)
    side.wait_stream(cur)
    sampler.set_stream(side.cuda_stream)
    fn()
    for t in tensors:
        t.record_stream(side)
    cur.wait_stream(side)


def trace_sampling(sampler: TraceSampler, zkets: torch.Tensor, dt: float, t_end: float, m: int, tol: float,
                   init_state: str = "singlet") -> torch.Tensor:
    """Trace sampling of the handle's Hamiltonian on device-resident sample
    vectors (samples x Z, complex128, CUDA): returns a (4, T) float64 tensor
    on the same device, rows P_S, P_T0, P_Tp, P_Tm, ordered after the
    caller's current stream's earlier work and before its later work
    (spc_trace_sampling_device); no host copies."""
    from .dynamics import num_time_points
    zk = _device_samples(zkets)
    T = num_time_points(dt, t_end)
    out = torch.empty(4 * T, dtype=torch.float64, device=zk.device)
    _ordered_call(sampler, zk.device, (zk, out), lambda: sampler.trace_sampling_device(
        zk.data_ptr(), zk.shape[0], dt, t_end, m, tol, out.data_ptr(), init_state))
    return out.view(4, T)


def trace_sampling_batch(sampler: TraceSampler, zkets_list, dt: float, t_end: float, m: int, tol: float,
                         init_state: str = "singlet", job_sys=None) -> torch.Tensor:
    """Batched trace sampling of the handle's batch store (build it with
    TraceSampler.build_h_batch) on device-resident sample tensors, one per
    job: returns a (jobs, 4, T) float64 tensor on the same device, ordered
    like trace_sampling (spc_trace_sampling_batch_device)."""
    from .dynamics import num_time_points
    zks = [_device_samples(z) for z in zkets_list]
    dev = zks[0].device
    flat = torch.cat([z.reshape(-1) for z in zks])
    T = num_time_points(dt, t_end)
    out = torch.empty(len(zks) * 4 * T, dtype=torch.float64, device=dev)
    _ordered_call(sampler, dev, (flat, out), lambda: sampler.trace_sampling_batch_device(
        flat.data_ptr(), [z.shape[0] for z in zks], dt, t_end, m, tol, out.data_ptr(), init_state, job_sys))
    return out.view(len(zks), 4, T)


__all__ = ["pack_params", "unpack_params", "yield_objective", "trace_sampling", "trace_sampling_batch"]
