"""Error statuses of the C ABI on the GPU: a non-finite charge density is
reported as PICGPU_NAN_DETECTED (not as a non-converged solve), and the
context stays usable for a finite one."""
import numpy as np
import pytest

from picfoam_gb300 import abi, cases
from picfoam_gb300.simulation import PicError

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precond", [abi.PRECOND_JACOBI, abi.PRECOND_MULTIGRID])
def test_nan_charge_density_is_reported(gpu, precond):
    case = cases.empty_case(n_cells=(8, 8, 8))
    case.cfg.pcg_precond = precond
    case.cfg.pcg_max_iter = 500
    sim = cases.build(case, backend=gpu)
    rho = np.full(512, 1e-6)
    rho[100] = np.nan
    with pytest.raises(PicError) as e:
        sim.solve_poisson(rho)
    assert e.value.status == abi.NAN_DETECTED and "not finite" in str(e.value)
    phi, st = sim.solve_poisson(np.full(512, 1e-6))
    assert np.all(np.isfinite(phi)) and st.pcg_residual_l2 <= case.cfg.pcg_tol
