"""The build entry point's smoke run: one frame of a 4,096-particle block on
the GPU, bit-exact with the oracle."""
from __future__ import annotations

import pytest

pytestmark = pytest.mark.gpu


def test_smoke_entry_point(native, capsys):
    import __graft_entry__

    __graft_entry__.smoke()
    assert "smoke ok" in capsys.readouterr().out
