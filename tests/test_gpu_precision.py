"""The precision study of the reduced forms (adfvm_gb300.studies: cylinder O-grid 256x128,
drag objective, FP32 and mixed against FP64), shortened to 200 steps: time-averaged drag and
its sensitivity to a source perturbation by the checkpointed adjoint sweep, both within 1e-5
relative of the FP64 run. (The full 2000-step study is run by bench.py and reported in its
line as precision_study.)"""
import pytest

pytestmark = pytest.mark.gpu


def test_precision_study_200_steps_within_1e5():
    from adfvm_gb300.studies import precision_study
    out = precision_study(nSteps=200, writeInterval=100)
    for prec in ('fp32', 'mixed'):
        for q in ('drag', 'sensitivity'):
            e = out['%s_%s_rel_err' % (prec, q)]
            assert e <= 1e-5, '%s %s: rel err %.3e' % (prec, q, e)
