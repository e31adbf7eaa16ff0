"""Device checks of the single-precision stand-ins for the reference's double
expressions (tracer_gb300/csrc/exact32.cuh) through tr_selftest: every result
must equal the double expression's float bit for bit. Case 0 covers all 2^32
inputs of the slab-test scale."""
import pytest

from tracer_gb300.native import selftest

pytestmark = pytest.mark.gpu

CASES = {1: "cross", 2: "normalize", 3: "cos", 4: "vector / float", 5: "shadow-ray length",
         6: "light pdf", 7: "disney fd90 / ss"}


def test_slab_scale_every_float(gpu):
    assert selftest(gpu, 0, 1 << 32) == 0


@pytest.mark.parametrize("which", sorted(CASES))
def test_certified_functions(gpu, which):
    for seed in (1, 2):
        assert selftest(gpu, which, 1 << 26, seed) == 0, CASES[which]
