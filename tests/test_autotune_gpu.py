"""The single-system tile autotuner on the GPU: it times every compiled shape of the
mixed direct kernel, installs the fastest per size and kind, and the tuned calls stay
within the mixed tolerance of the FP64 oracle (rms <= 1e-6, max <= 1e-3)."""
import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu


def test_tune_direct_installs_winners(lib, cuda):
    from gravhopper_gb300 import _jbgrav, autotune, ics
    sizes = (3000, 30000)
    try:
        res = autotune.tune_direct(sizes=sizes, kinds=("force", "step"), use_cache=False)
        nshape = lib.gh_direct_num_shapes()
        for kind in ("force", "step"):
            for n in sizes:
                best, ms = res[kind][n]
                assert sorted(ms) == list(range(nshape))
                assert all(t > 0 for t in ms.values())
                assert ms[best] == min(ms.values())
                assert autotune.shape_for(n, kind) == best
        ic = ics.plummer(3000, seed=31)
        ref = oracle.direct_summation(ic["pos"], ic["mass"], 5e-5)
        got = _jbgrav.direct_summation_mixed(ic["pos"], ic["mass"], 5e-5)
        r = np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1)
        assert np.sqrt(np.mean(r * r)) <= 1e-6 and r.max() <= 1e-3
    finally:
        autotune.clear_direct()
