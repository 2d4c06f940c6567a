"""The allocation-free evaluation entry point against the allocating one.

cedar_eval_dev_noalloc serves callers that may not allocate device memory when
they call (real-time loops that ban allocation after set-up, hosts whose device
memory another runtime's pool allocator reserved up front): its scratch is a
fixed per-device array inside the library.  This test drives both entry points
through the C ABI on the same device buffers and checks that the results are the
same bits (both run the same kernels; only the scratch differs), on two calls in
a row with different states, so stale scratch would show.  One case has supply
rails longer than the long-row threshold, so the partial-sum region of the
scratch is exercised as well as the device outputs.
"""
import ctypes as C

import numpy as np
import pytest

from tests import circuits as K

pytestmark = pytest.mark.gpu


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _scratch(lib, handle):
    n_out, n_part, limit = C.c_int64(), C.c_int64(), C.c_int64()
    rc = lib.cedar_eval_scratch(handle, C.byref(n_out), C.byref(n_part), C.byref(limit))
    assert rc == 0
    return n_out.value, n_part.value, limit.value


def _limit(lib):
    limit = C.c_int64()
    assert lib.cedar_eval_scratch(None, None, None, C.byref(limit)) == 0
    return limit.value


def _flat(pkg, case):
    if case == "inverter_chain":
        return pkg.generators.inverter_chain(9).flatten()
    if case == "long_rails":
        return pkg.generators.inverter_chain(100).flatten()
    return K.mixed(pkg).flatten()


@pytest.mark.parametrize("case", ["inverter_chain", "mixed", "long_rails"])
def test_noalloc_eval_matches_allocating_eval(gpu, pkg, case):
    import torch
    flat = _flat(pkg, case)
    sys_ = pkg.System(flat)
    lib = sys_.lib
    n_out, n_part, limit = _scratch(lib, sys_.handle)
    assert 0 < n_out + n_part <= limit
    if case == "long_rails":
        # the 100-stage chain's supply rows (200 entries) exceed the long-row threshold
        assert n_part > 0
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
        assert np.array_equal(Fn, Fr) and np.array_equal(Jn, Jr)


def test_noalloc_allocates_nothing(gpu, pkg):
    """100 calls leave the device's free memory unchanged (after one warm-up call,
    which loads the kernels and looks up the scratch address)."""
    import torch
    sys_ = pkg.System(pkg.generators.inverter_chain(100).flatten())
    lib = sys_.lib
    dev = torch.device("cuda:0")
    x = torch.rand(sys_.n, dtype=torch.float64, device=dev) * 1.8
    F = torch.empty(sys_.n, dtype=torch.float64, device=dev)
    J = torch.empty(sys_.nnz_j, dtype=torch.float64, device=dev)
    call = lambda: pkg.abi.check(lib.cedar_eval_dev_noalloc(sys_.handle, _ptr(x), None, 1e-9, 1e12, _ptr(F), _ptr(J),
                                                            None))
    call()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(100):
        call()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert bool(torch.isfinite(F).all()) and bool(torch.isfinite(J).all())


def test_noalloc_rejects_oversized_circuit(gpu, pkg):
    """A circuit whose scratch need exceeds the fixed array gets a clear error
    from the host-side size check, before anything is launched."""
    import torch
    lib = pkg.load_library()
    limit = _limit(lib)
    c = pkg.Circuit()
    c.V("V1", "a", "0", dc=1.0)
    n_caps = limit // 3 + 1000
    for k in range(n_caps):
        c.C(f"C{k}", "a", "0", 1e-15)
    sys_ = pkg.System(c)
    n_out, n_part, limit2 = _scratch(lib, sys_.handle)
    assert limit2 == limit and n_out + n_part > limit
    dev = torch.device("cuda:0")
    # valid, correctly sized buffers, so that the call is well formed apart from the size
    x = torch.zeros(sys_.n, dtype=torch.float64, device=dev)
    F = torch.zeros(sys_.n, dtype=torch.float64, device=dev)
    J = torch.zeros(sys_.nnz_j, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    buf = C.create_string_buffer(256)
    rc = lib.cedar_eval_dev_noalloc(sys_.handle, _ptr(x), None, 0.0, 0.0, _ptr(F), _ptr(J), None)
    assert rc == -1
    lib.cedar_last_error(buf, 256)
    assert f"at most {limit}".encode() in buf.value
