"""The allocation-free evaluation entry point against the allocating one.

cedar_eval_dev_noalloc serves callers that may not allocate device memory when
they call (real-time loops that ban allocation after set-up, hosts whose device
memory another runtime's pool allocator reserved up front): its scratch is a
fixed per-device array inside the library.  This test drives both
entry points through the C ABI on the same device buffers and checks that the
results agree within the evaluation tolerance of the other GPU tests, on two calls
in a row (the second with a different state, so stale scratch would show).
"""
import ctypes as C

import numpy as np
import pytest

from tests import circuits as K

pytestmark = pytest.mark.gpu

RTOL_EVAL = 1e-12


def _ptr(t):
    return C.c_void_p(t.data_ptr())


@pytest.mark.parametrize("case", ["inverter_chain", "mixed"])
def test_noalloc_eval_matches_allocating_eval(gpu, pkg, case):
    import torch
    flat = (pkg.generators.inverter_chain(9) if case == "inverter_chain" else K.mixed(pkg)).flatten()
    sys_ = pkg.System(flat)
    lib = sys_.lib
    n, nj = sys_.n, sys_.nnz_j
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(17)
    for call in range(2):
        x = torch.tensor(rng.uniform(-0.2, 1.8, n), dtype=torch.float64, device=dev)
        xd = torch.tensor(rng.normal(0, 1e9, n), dtype=torch.float64, device=dev)
        t, cj = 0.2e-9 * (call + 1), 10.0 ** (10 + call)
        F_ref = torch.zeros(n, dtype=torch.float64, device=dev)
        J_ref = torch.zeros(nj, dtype=torch.float64, device=dev)
        F_new = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
        J_new = torch.full((nj,), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        pkg.abi.check(lib.cedar_eval_dev(sys_.handle, _ptr(x), _ptr(xd), t, cj, _ptr(F_ref), _ptr(J_ref)))
        stream = torch.cuda.current_stream().cuda_stream
        pkg.abi.check(lib.cedar_eval_dev_noalloc(sys_.handle, _ptr(x), _ptr(xd), t, cj, _ptr(F_new), _ptr(J_new),
                                                 C.c_void_p(stream)))
        torch.cuda.synchronize()
        Fr, Fn = F_ref.cpu().numpy(), F_new.cpu().numpy()
        Jr, Jn = J_ref.cpu().numpy(), J_new.cpu().numpy()
        assert np.all(np.isfinite(Fn)) and np.all(np.isfinite(Jn))
        assert np.all(np.abs(Fn - Fr) <= RTOL_EVAL * np.abs(Fr) + 1e-300)
        assert np.all(np.abs(Jn - Jr) <= RTOL_EVAL * np.abs(Jr) + 1e-300)


def test_noalloc_rejects_oversized_circuit(gpu, pkg):
    """A circuit whose device outputs exceed the fixed scratch gets a clear error
    from the host-side size check, before anything is launched."""
    import torch
    limit = 262144
    n_caps = 100000                      # 3 outputs each, plus 4 for the source
    n_out = 3 * n_caps + 4
    assert n_out > limit + 30000         # well past the limit
    c = pkg.Circuit()
    c.V("V1", "a", "0", dc=1.0)
    for k in range(n_caps):
        c.C(f"C{k}", "a", "0", 1e-15)
    sys_ = pkg.System(c)
    dev = torch.device("cuda:0")
    # valid, correctly sized buffers, so that the call is well formed apart from the size
    x = torch.zeros(sys_.n, dtype=torch.float64, device=dev)
    F = torch.zeros(sys_.n, dtype=torch.float64, device=dev)
    J = torch.zeros(sys_.nnz_j, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    buf = C.create_string_buffer(256)
    rc = sys_.lib.cedar_eval_dev_noalloc(sys_.handle, _ptr(x), None, 0.0, 0.0, _ptr(F), _ptr(J), None)
    assert rc == -1
    sys_.lib.cedar_last_error(buf, 256)
    assert b"at most 262144" in buf.value
