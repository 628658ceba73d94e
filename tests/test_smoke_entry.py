"""__graft_entry__.smoke() end to end (one small solve on cuda:0 against the oracle)."""
import pytest

pytestmark = pytest.mark.gpu


def test_smoke(built):
    import __graft_entry__ as g
    g.smoke()
