"""The random-access peak entry point (roofline denominator of the search)."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["gather", "cas"])
def test_random_access_peak_is_measured(engine, kind):
    r = engine.random_access_peak(kind, buffer_bytes=1 << 30)
    assert r["ms"] > 0
    # Far below the streaming copy rate of the device, far above zero.
    assert 50.0 < r["gbs"] < 20000.0, r
