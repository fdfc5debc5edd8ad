"""The oracle's pressure multigrid (CPU, no GPU): semi-coarsening keeps the
BiCGSTAB iteration count low on anisotropic grids, and isotropic grids keep
full 2x2 coarsening."""
import pytest

from immerseflow_gb300 import _capi as capi
from immerseflow_gb300 import cases


def case(nx, ny):
    return cases.external(nx, ny, 12.0, 8.0, 4.0, 4.0, 0.5, 0.3, 10.0, 130.0, 4e-3, capi.PREC_FP64)


@pytest.mark.parametrize("nx,ny", [(64, 315), (481, 73), (96, 64)])
def test_iterations_bounded_on_anisotropic_grids(oracle, nx, ny):
    o = oracle.method(*case(nx, ny))
    o.step(2)
    assert o.stats().last_ppe_iters <= 12


def test_level_counts():
    # isotropic 96x64 on 12x8: 96x64 -> 48x32 -> 24x16 -> 12x8 -> 6x4 (five levels)
    import _oracle
    o = _oracle.Oracle().method(*case(96, 64))
    assert o.levels() == 5
    # 64x315 (cells 6.4:1): y-only coarsening first, so more levels than 2x2 coarsening would give
    o = _oracle.Oracle().method(*case(64, 315))
    assert o.levels() == 7
