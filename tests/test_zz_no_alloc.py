"""spc_build_h_noalloc: the Hamiltonian build for callers that cannot allocate
device memory (a fixed device-memory pool, plugins that only pass their own
buffers). It keeps its scratch in a static device array, so it is checked
here through the C ABI against the allocating entry point (spc_build_h +
spc_get_h) on consecutive calls that reuse that array.

This file is collected last on purpose: a run that stops at the first
failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

from spin_dynamics_gb300 import _native as nat
from spin_dynamics_gb300 import workloads as W
from spin_dynamics_gb300.dynamics import make_system
from spin_dynamics_gb300.spinsys import Electron, SysParam

pytestmark = pytest.mark.gpu


def _noalloc(sysp, B, mode, cap, fill=0):
    import torch

    s, keep = make_system(sysp, B)
    n = sysp.N
    rp = torch.full((n + 1,), fill, dtype=torch.int32, device="cuda:0")
    col = torch.full((cap,), fill, dtype=torch.int32, device="cuda:0")
    val = torch.full((2 * cap,), float(fill), dtype=torch.float64, device="cuda:0")
    n_out, nnz_out = C.c_int32(), C.c_int64()
    stream = torch.cuda.current_stream().cuda_stream
    rc = nat.lib().spc_build_h_noalloc(C.byref(s), mode, C.c_void_p(rp.data_ptr()),
                                       C.c_void_p(col.data_ptr()), C.c_void_p(val.data_ptr()), cap,
                                       C.byref(n_out), C.byref(nnz_out), C.c_void_p(stream))
    return rc, n_out.value, nnz_out.value, rp, col, val


def _expected(sampler, sysp, B, mode_name):
    sampler.build_h(sysp, B, mode_name)
    return sampler.get_h()


def test_noalloc_build_matches_allocating_build_on_consecutive_calls(sampler):
    large, B = W.large_pair()
    small = W.small_pair()
    cases = [(large, B, nat.SPC_H_GENERAL, "general"),
             (small, 0.05, nat.SPC_H_REFERENCE, "reference"),
             (large, B, nat.SPC_H_GENERAL, "general")]
    for sysp, field, mode, name in cases:
        rp_e, col_e, val_e = _expected(sampler, sysp, field, name)
        rc, n, nnz, rp, col, val = _noalloc(sysp, field, mode, len(col_e))
        nat.check(rc)
        assert n == sysp.N and nnz == len(col_e)
        assert np.array_equal(rp.cpu().numpy(), rp_e)
        assert np.array_equal(col.cpu().numpy(), col_e)
        assert np.array_equal(val.cpu().numpy().view(np.complex128), val_e)


def test_noalloc_rejects_sizes_beyond_its_scratch(sampler):
    # 21 spin-1/2 nuclei: 4 * 2^21 rows, above the 2^20 rows of the scratch
    big = SysParam(e1=Electron(g_I=[2] * 11, A=[np.eye(3) * 0.1] * 11),
                   e2=Electron(g_I=[2] * 10, A=[np.eye(3) * 0.1] * 10))
    rc, *_ = _noalloc(big, 0.05, nat.SPC_H_REFERENCE, 8)
    assert rc == nat.SPC_ERR_ARG
    assert b"scratch" in nat.lib().spc_last_error()
    # too small an output capacity is refused from the closed-form count,
    # before any launch: every output buffer keeps its contents
    rc, n, nnz, rp, col, val = _noalloc(W.small_pair(), 0.05, nat.SPC_H_REFERENCE, 10, fill=-7)
    assert rc == nat.SPC_ERR_ARG and nnz > 10 and n == W.small_pair().N
    assert bool((rp == -7).all()) and bool((col == -7).all()) and bool((val == -7.0).all())


def test_noalloc_general_build_of_a_symmetry_block(sampler):
    # a block with effective nuclei of multiplicity 5 and 3 (entry tables of
    # 48 g elements per nucleus) through the table-driven general fill
    g1h, g14n = 0.26752218708, 0.0193297792
    blk = SysParam(e1=Electron(g_I=[5, 3, 2], A=[np.diag([0.3, 0.3, 0.5]), np.eye(3) * 0.2, np.eye(3) * 0.7],
                               gamma_I=[g1h, g14n, g1h]),
                   e2=Electron(g_I=[3, 2], A=[np.eye(3) * 0.4, np.diag([0.1, 0.2, 0.9])], gamma_I=[g14n, g1h]),
                   J=0.01, kS=0.02, kT=0.01)
    field = np.array([0.02, -0.03, 0.05])
    rp_e, col_e, val_e = _expected(sampler, blk, field, "general")
    for _ in range(2):
        rc, n, nnz, rp, col, val = _noalloc(blk, field, nat.SPC_H_GENERAL, len(col_e))
        nat.check(rc)
        assert n == blk.N and nnz == len(col_e)
        assert np.array_equal(rp.cpu().numpy(), rp_e)
        assert np.array_equal(col.cpu().numpy(), col_e)
        assert np.array_equal(val.cpu().numpy().view(np.complex128), val_e)
