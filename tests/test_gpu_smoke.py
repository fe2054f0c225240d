"""The package's smoke entry point (one small KB gridding call and one drop-in
linear gridding call on cuda:0, each checked against the oracle) runs clean."""

import pytest


@pytest.mark.gpu
def test_smoke_entry_point(native):
    import __graft_entry__

    __graft_entry__.smoke()
