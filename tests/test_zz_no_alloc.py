"""scihpc_lsf_integrals_noalloc: the enclosed mass and volume for callers that cannot
allocate device memory (code running inside someone else's CUDA graph capture, plugins
whose host application owns all device memory, loops that must not touch the allocator).
Its scratch lives in a static device array, so it must agree with the context-based
scihpc_lsf_integrals -- on two calls in a row, since the array keeps the previous call's
contents -- and must reject grids larger than that array.

Collected last on purpose (file name): if it fails, a run that stops at the first failure
has already run every other test."""
import numpy as np
import pytest

import oracle as O
from tests.helpers import bubble_phi, smooth_field

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

TOL = 1e-13   # the tolerance of the integrals in test_gpu_kernels.py


def _cases():
    g2 = O.Grid(2, (24, 40), (0.0, 0.0), (1.0, 2.0))
    phi2 = O.Checker("port").bc_fill(g2, 0, [1] * 6, [0.0] * 6, bubble_phi(g2, (0.5, 0.9), 0.3))
    g3 = O.Grid(3, (12, 14, 10), (0.0, 0.0, 0.0), (1.0, 2.0, 1.5))
    phi3 = 0.1 * smooth_field(g3, np.random.default_rng(11))
    return [(g2, phi2), (g3, phi3)]


@pytest.mark.parametrize("case", [0, 1])
def test_noalloc_matches_context_entry_point(case):
    from scihpc_gb300 import Grid, Workspace
    from scihpc_gb300.native import lsf_integrals_noalloc
    g, phi = _cases()[case]
    ng = Grid(g.ndim, tuple(g.n), tuple(g.lo), tuple(g.hi))
    h = min(g.spacing())
    prm = [1.5 * h, 0.001, 0.01, 0.0]
    d = torch.from_numpy(np.ascontiguousarray(phi)).cuda()
    ref = Workspace(ng).lsf_integrals(prm, d)
    for call in range(2):
        out = lsf_integrals_noalloc(ng, prm, d)
        for q in range(2):
            assert abs(out[q] - ref[q]) <= TOL * abs(ref[q]), (call, q, out, ref)


def test_noalloc_rejects_oversize_grid():
    from scihpc_gb300 import Grid, ScihpcError
    from scihpc_gb300.native import lsf_integrals_noalloc
    g = Grid(3, (200, 200, 200), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0))
    phi = torch.zeros(1, dtype=torch.float64, device="cuda")   # never read: the size check comes first
    with pytest.raises(ScihpcError, match="static scratch"):
        lsf_integrals_noalloc(g, [0.01, 0.001, 0.01, 0.0], phi)
