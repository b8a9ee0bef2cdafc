"""The allocation-free integrate entry point (mkpp_gpu_integrate_noalloc).

Some host models must not allocate device memory where they call the
chemistry: their own pool allocator owns the free device memory, or their
time loop avoids cudaMalloc/cudaFree because those synchronise the whole
device.  This entry point keeps its scratch in a static device array of the
library instead.  The test calls it through the C ABI on two calls in a row
and checks each against the workspace-based entry point on the same inputs:
the second call takes other cells than the first, so a result that leaned on
what the first call left in the shared array would differ.  It is collected
last so that a failure here comes after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_matches_workspace_entry_point(built_libs):
    import torch

    from mkpp_gb300 import workloads
    from mkpp_gb300.api import DeviceSolver, load_library

    lib = load_library("saprc99")
    s = DeviceSolver("saprc99")
    n = 512
    w = workloads.make("saprc99", 2 * n)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731

    for call in range(2):
        cells = slice(call * n, (call + 1) * n)
        conc0 = d(w.conc[:, cells])
        ktab, st0 = s.rate_constants(conc0, d(w.temp[cells]), d(w.rho[cells]), d(w.rh[cells]), None,
                                     d(w.param[:, cells]))
        torch.cuda.synchronize()

        # Existing entry point (plain form, caller-provided workspace).
        ref = conc0.clone()
        rst = st0.clone()
        racc = torch.zeros(n, dtype=torch.int32, device="cuda")
        rrej = torch.zeros_like(racc)
        s.integrate_k(ref, ktab, w.dt, mode="plain", status=rst, accepted=racc, rejected=rrej)
        torch.cuda.synchronize()

        out = conc0.clone()
        ost = st0.clone()
        oacc = torch.zeros(n, dtype=torch.int32, device="cuda")
        orej = torch.zeros_like(oacc)
        rc = lib.mkpp_gpu_integrate_noalloc(C.c_size_t(n), p(out), p(ktab), C.c_size_t(0), 1, C.c_double(w.dt),
                                            C.c_double(s.default_seed), 20000, p(ost), p(oacc), p(orej), stream)
        assert rc == 0, rc
        torch.cuda.synchronize()
        # Bit for bit (a non-finite cell compares as non-finite on both sides).
        assert torch.equal(torch.nan_to_num(out, nan=1.25e300), torch.nan_to_num(ref, nan=1.25e300)), f"call {call}"
        assert torch.equal(ost, rst) and torch.equal(oacc, racc) and torch.equal(orej, rrej), f"call {call}"


def test_noalloc_rejects_more_cells_than_its_scratch(built_libs):
    from mkpp_gb300.api import load_library

    lib = load_library("saprc99")
    dummy = C.c_void_p(256)  # never dereferenced: the size check comes first
    rc = lib.mkpp_gpu_integrate_noalloc(C.c_size_t(1025), dummy, dummy, C.c_size_t(0), 1, C.c_double(600.0),
                                        C.c_double(1e-6), 20000, None, None, None, None)
    assert rc == -103
