"""The autotuner times every ogs variant and its winner reproduces the reference's
bits (GPU)."""
import numpy as np
import pytest
import torch

from streamparanumal_gb300 import autotune, capi
from streamparanumal_gb300 import ogs as O

pytestmark = pytest.mark.gpu


def test_tune_and_apply_small_box(cuda, orc, tmp_path):
    saved = {k: capi.tune_get(v) for k, v in autotune.KNOBS.items()}
    try:
        res = autotune.tune_ogs(4, 3, perm_seed=5, reps=2)
        best = res["best"]
        assert set(best) >= {"order", "rows", "page_shift", "kernel_gs", "kernel_gather",
                             "kernel_scatter", "block_nnz"}
        # grouped plans (2, plus 64-entry pages at p = 3, plus the renumbered walk,
        # plus the three breadth-first ones as chains of balls) x (6 + 4 + 6) kernels
        # and the walk-ordered column-major scatter under the six breadth-first ones,
        # the breadth-first CSR plan x (6 + 2 + 6), the row-order CSR plan with block
        # kernels and the column-major scatter too (7 + 4 + 7), and block kernels at
        # block_nnz 1024 (3); then the gather+scatter walks x their kernels
        assert len(res["candidates"]) == 112 + 6 + 14 + 18 + 3
        assert len(res["gs_walks"]) in (0, len(autotune.GS_WALK_KERNELS) * len(autotune.gs_walks(3)))
        table = {}
        autotune.record(table, res)
        path = tmp_path / "t.json"
        autotune.save_table(table, path)
        cfg = autotune.apply(3, True, autotune.load_table(path))
        assert cfg == best
        ids = O.box_hex_ids(4, 4, 4, 3, 5)
        ref = orc.ogs_setup(ids.copy(), kind=1, unique=True)
        h = O.ogs_t()
        h.Setup(ids.size, ids, unique=True)
        q = orc.uniform(ids.size, 4)
        dq = torch.from_numpy(q).cuda()
        h.GatherScatter(dq, 1, O.Add, O.Sym)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(
            dq.cpu().numpy(),
            orc.gather_scatter(ref["rsT"], ref["ciT"], ref["rsT"], ref["ciT"], q))
    finally:
        autotune._set(saved)
