"""The integer-pipe double division and square root used by the FP64 step
must agree bit for bit with the hardware IEEE operations (the exact build's
forms) or lie within one neighbour of them (the FMA build's faithful forms),
and the exponent-test pressure floor and limiter sign test with the products
they skip."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [0, 1, 2, 3, 4], ids=["any-bits", "near-1", "wide", "near-boundary", "zeros"])
@pytest.mark.parametrize("op", [0, 1, 2, 3, 4, 5, 6, 7],
                         ids=["div", "sqrt", "pressure-floor", "limiter-sign", "div-faithful", "sqrt-faithful",
                              "f32-div-faithful", "f32-sqrt-faithful"])
def test_emulated_matches_hardware(e2d, op, mode):
    bad, first, _ = e2d.selftest_arith(op, mode, 1 << 26, seed=12345 + 17 * mode + op)
    assert bad == 0, f"{bad} mismatches; first (a, b, emulated, hardware) = {first}"


def test_emulated_rates_reported(e2d):
    for op in (0, 1, 4, 5):
        bad, _, (em, na) = e2d.selftest_arith(op, 1, 1 << 20, seed=7, rates=True)
        assert bad == 0 and em > 0 and na > 0
        print(f"op {op}: emulated {em / 1e9:.1f} G/s, hardware {na / 1e9:.1f} G/s")
