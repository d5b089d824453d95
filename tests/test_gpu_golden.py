"""The reference's own kernel, run live: its HD must equal the oracle's and
the CUDA path's on every golden case, for both structuring elements."""
import os
import sys

import pytest
import torch

pytestmark = pytest.mark.gpu
sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))

from cases import cases  # noqa: E402
from oracle import ref_kernel  # noqa: E402


@pytest.mark.skipif(not (ref_kernel.available("se18") and ref_kernel.available("se6")),
                    reason="reference kernel PTX not built (needs the reference sources at build time)")
@pytest.mark.parametrize("se", ["se6", "se18"])
def test_reference_kernel_matches(ctx, oracle, se):
    for name, make in cases().items():
        a, b = make()
        ref = ref_kernel.ref_hd(a, b, se)
        o = oracle.forbench(a, b, se)
        g = ctx.compute(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), se)
        assert ref == o["hd"] == g["hd"], (name, se, ref, o["hd"], g["hd"])
