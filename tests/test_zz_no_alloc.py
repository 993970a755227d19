"""The no-allocation direct-sum entry point, through the C ABI.

gh_direct_mixed_noalloc is for callers that cannot let the library allocate device
memory (an application that owns all device memory through its own pool, or a
stepping loop that must not call cudaMalloc/cudaFree because they can synchronise the
device).  Its scratch is a fixed array inside the library, so this checks two calls
in a row against the allocating entry point gh_direct_dev (mixed precision, within
1e-6) and against the FP64 oracle, within the mixed form's tolerance (rms 1e-6 with
softening, 1e-5 with eps = 0, the variant that gives a coincident pair no term), and
that sizes beyond the fixed limit are refused.  Collected last so that a stop-at-first-failure run has run
every other test first.
"""
import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu

MIXED_RMS_TOL = 1e-6
MIXED_MAX_TOL = 1e-3
# Without softening the closest pairs' FP32 offsets dominate their forces; the mixed
# form's stated tolerance against FP64 there is rms 1e-5 (as for the other eps = 0 tests).
MIXED_RMS_TOL_EPS0 = 1e-5
NOALLOC_MAX_N = 65536


def _rel(a, b):
    r = np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)
    return float(np.sqrt(np.mean(r * r))), float(r.max())


@pytest.mark.parametrize("eps", [5e-5, 0.0])
def test_no_alloc_matches_allocating_entry_point_and_oracle(lib, cuda, eps):
    import torch

    from gravhopper_gb300 import _capi, ics
    for n, seed in ((5000, 1), (NOALLOC_MAX_N, 2)):
        ic = ics.plummer(n, seed=seed)
        x = torch.from_numpy(ic["pos"]).to(cuda)
        m = torch.from_numpy(ic["mass"]).to(cuda)
        stream = torch.cuda.current_stream().cuda_stream
        ref = torch.empty((n, 3), dtype=torch.float64, device=cuda)
        _capi.check(lib.gh_direct_dev(x.data_ptr(), m.data_ptr(), n, None, 0, eps, _capi.GH_PREC_MIXED,
                                      ref.data_ptr(), stream))
        ref_h = ref.cpu().numpy()
        exact = oracle.direct_summation(ic["pos"], ic["mass"], eps)
        for call in range(2):
            out = torch.full((n, 3), float("nan"), dtype=torch.float64, device=cuda)
            _capi.check(lib.gh_direct_mixed_noalloc(x.data_ptr(), m.data_ptr(), n, eps, out.data_ptr(), stream))
            got = out.cpu().numpy()
            assert np.isfinite(got).all(), (n, eps, call)
            assert _rel(got, ref_h)[0] <= MIXED_RMS_TOL, (n, eps, call)
            rms, mx = _rel(got, exact)
            tol = MIXED_RMS_TOL if eps > 0 else MIXED_RMS_TOL_EPS0
            assert rms <= tol and mx <= MIXED_MAX_TOL, (n, eps, call, rms, mx)


def test_no_alloc_refuses_oversize(lib, cuda):
    import torch

    from gravhopper_gb300 import _capi
    n = NOALLOC_MAX_N + 1
    x = torch.zeros((n, 3), dtype=torch.float64, device=cuda)
    m = torch.ones(n, dtype=torch.float64, device=cuda)
    out = torch.empty((n, 3), dtype=torch.float64, device=cuda)
    rc = lib.gh_direct_mixed_noalloc(x.data_ptr(), m.data_ptr(), n, 5e-5, out.data_ptr(),
                                     torch.cuda.current_stream().cuda_stream)
    assert rc == _capi.GH_ERR_ARG
    assert b"limit" in lib.gh_last_error()
