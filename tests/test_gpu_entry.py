"""The entry point's smoke check (one small force evaluation and two steps on
cuda:0 against the oracle) runs as part of the GPU suite."""
import pytest

import __graft_entry__

pytestmark = pytest.mark.gpu


def test_smoke_entry_point(capsys):
    __graft_entry__.smoke()
    assert "smoke ok" in capsys.readouterr().out
