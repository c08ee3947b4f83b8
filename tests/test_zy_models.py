"""The non-default DCS models on the GPU (struct pumas_physics_settings,
pumas.h:742-771): KKP and ABB bremsstrahlung, KKP pair production, BM and
BBKS photonuclear interactions (pumas_gb300/csrc/gp_models.cuh, the code the
CPU oracle runs too). The golden cases models_* of tests/cases.py, made by
the reference with physics dumps of those models, run through the same check
as the default models' cases. This file is collected after the other GPU
test files but before the allocation-free entry point's.
"""
import numpy as np
import pytest

from cases import CASES, has_models
from test_gpu_parity import golden_check

pytestmark = pytest.mark.gpu

MODEL_CASES = sorted(n for n in CASES if has_models(n))


@pytest.mark.parametrize("name", MODEL_CASES)
def test_gpu_models_match_reference_golden(request, name):
    good, n = golden_check(request, name)
    assert good >= 0.999 * n    # all of them so far


def test_model_physics_load(request):
    from conftest import case_physics
    for name in MODEL_CASES:
        physics = case_physics(request, name)
        assert physics.n_materials == 4
    assert np.isfinite(physics.mass)
