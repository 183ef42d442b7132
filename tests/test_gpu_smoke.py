"""The build-and-smoke entry point runs end to end on the GPU."""
import pytest

pytestmark = pytest.mark.gpu


def test_smoke_entry_point(capsys):
    import __graft_entry__ as g
    g.smoke()
    assert "smoke ok" in capsys.readouterr().out
