"""A molecule of the large-molecule workload (1000-2000 atoms) on the GPU.

The reference itself was run on it (tests/golden/large_ref.json, made by
tests/golden/make_large_refs.py): with its Anderson mixer and 300
iterations its SCF does not converge.  The engine, given the same budget,
must say the same (status NOT_CONVERGED with a SCFConvergenceWarning) and
return finite numbers, running every large-molecule kernel on the way:
the blocked Cholesky over the whole GPU, the blocked cluster
tridiagonalisation and the shared-memory opt-in of the eigenvector
kernels at more than 3000 orbitals."""
import json
import warnings

import numpy as np
import pytest
import torch

from dxtb_gb300 import _lib, molgen
from tests.helpers import GOLDEN

pytestmark = pytest.mark.gpu

TIGHT = {"exclude": ["disp"], "maxiter": 300, "x_atol": 1e-10, "x_atol_max": 1e-10}


def test_large_molecule_agrees_with_the_reference_on_convergence():
    from dxtb_gb300 import GFN1Calculator, SCFConvergenceWarning

    refs = json.loads((GOLDEN / "large_ref.json").read_text())
    k = min(refs, key=lambda x: refs[x]["natom"])
    ref = refs[k]
    num, pos = molgen.c5_large(16)[int(k)]
    assert len(num) == ref["natom"]
    calc = GFN1Calculator(torch.as_tensor(num), opts=TIGHT)
    with warnings.catch_warnings(record=True) as caught:
        warnings.simplefilter("always")
        res = calc.singlepoint(torch.tensor(pos, device="cuda"))
    converged = res.status[0] & _lib.MOL_NOT_CONVERGED == 0
    assert res.status[0] & ~_lib.MOL_NOT_CONVERGED == 0
    assert converged == ref["converged"]
    if not converged:
        assert any(issubclass(w.category, SCFConvergenceWarning) for w in caught)
    assert np.isfinite(res.energy.item()) and np.isfinite(res.charges.cpu().numpy()).all()
