"""The L2 eviction priorities of the stencil bulk copies (CITCOM_GPU_L2HINT,
CITCOM_GPU_L2KEEP_MB, read when a handle is created) only decide which lines
the L2 evicts first.  A mixed solve without them, with the default policy
(finest level evict_first, 64 MB of the coarser tile levels evict_last) and
with every coarser tile level kept, takes the same iterations and gives
bit-identical U and P."""
import os

import numpy as np
import pytest

from tests.test_gpu_residual_rule import box_case, seeded_T0

pytestmark = pytest.mark.gpu


def test_l2_priorities_leave_results_bit_identical():
    import citcomcu_gb300 as cg
    cg.build()
    case = box_case(32)
    T0 = seeded_T0(case)
    out = {}
    for name, env in (("none", {"CITCOM_GPU_L2HINT": "0"}), ("default", {}),
                      ("keep_all", {"CITCOM_GPU_L2KEEP_MB": "100000"})):
        old = {k: os.environ.get(k) for k in ("CITCOM_GPU_L2HINT", "CITCOM_GPU_L2KEEP_MB")}
        for k in old:
            os.environ.pop(k, None)
        os.environ.update(env)
        try:
            s = cg.Solver(cg.Config.like(case, precision=cg.MIXED))
        finally:
            for k, v in old.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v
        f = s.fine
        U, P = np.zeros(f["neq"]), np.zeros(f["nel"])
        s.general_stokes_solver(T0, U, P)
        st = s.stats()
        out[name] = (U, P, st["uzawa"], st["mg_passes"])
        s.close()
    ref = out["none"]
    for name in ("default", "keep_all"):
        U, P, uz, mg = out[name]
        print(name, uz, mg, ref[2], ref[3])
        assert uz == ref[2] and mg == ref[3]
        assert np.array_equal(U, ref[0]) and np.array_equal(P, ref[1])
