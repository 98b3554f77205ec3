"""The precision study of the reduced forms (adfvm_gb300.studies: cylinder O-grid 256x128,
drag objective, FP32 and mixed against FP64): time-averaged drag and its sensitivity to a
source perturbation by the checkpointed adjoint sweep. Shortened to 200 steps, both reduced
forms are within 1e-5 relative of the FP64 run; over the full 2000 steps the mixed form (FP32
gauge-offset records and face arithmetic, FP64 state and adjoints) is, while the FP32 form,
whose state itself is rounded to floats every stage, is within 5e-5."""
import pytest

pytestmark = pytest.mark.gpu


def test_precision_study_200_steps_within_1e5():
    from adfvm_gb300.studies import precision_study
    out = precision_study(nSteps=200, writeInterval=100)
    for prec in ('fp32', 'mixed'):
        for q in ('drag', 'sensitivity'):
            e = out['%s_%s_rel_err' % (prec, q)]
            assert e <= 1e-5, '%s %s: rel err %.3e' % (prec, q, e)


def test_precision_study_2000_steps():
    from adfvm_gb300.studies import precision_study
    out = precision_study(nSteps=2000, writeInterval=100)
    for q in ('drag', 'sensitivity'):
        e = out['mixed_%s_rel_err' % q]
        assert e <= 1e-5, 'mixed %s: rel err %.3e' % (q, e)
        e = out['fp32_%s_rel_err' % q]
        assert e <= 5e-5, 'fp32 %s: rel err %.3e' % (q, e)
