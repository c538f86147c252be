"""scihpc_lsf_integrals_noalloc: the enclosed mass and volume for callers that cannot
allocate device memory (plugins whose host application owns all device memory through its
own pool, real-time loops that must not touch the allocator).  Its scratch lives in a
static device array, so it must agree with the context-based scihpc_lsf_integrals -- on
two calls in a row, since the array keeps the previous call's contents, and on grids that
fill the array exactly -- and must reject grids larger than that array.

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
    # grids whose ghosted size is exactly the scratch maximum (1,048,576 cells): 1024 x 1024
    # and 64 x 128 x 128 ghosted; the partial sums sit right after the product field
    g2m = O.Grid(2, (1018, 1018), (0.0, 0.0), (1.0, 1.0))
    phi2m = bubble_phi(g2m, (0.45, 0.55), 0.3)
    g3m = O.Grid(3, (58, 122, 122), (0.0, 0.0, 0.0), (0.5, 1.0, 1.0))
    x, y, z = np.meshgrid(*[g3m.lo[a] + (np.arange(g3m.shape[a]) - 2.5) * g3m.spacing()[a] for a in range(3)],
                          indexing="ij")
    phi3m = 0.3 - np.sqrt((x - 0.25) ** 2 + (y - 0.5) ** 2 + (z - 0.45) ** 2)
    assert np.prod(g2m.shape) == 1 << 20 and np.prod(g3m.shape) == 1 << 20
    return [(g2, phi2), (g3, phi3), (g2m, phi2m), (g3m, phi3m)]


@pytest.mark.parametrize("case", [0, 1, 2, 3])
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
