"""The build entry point's smoke check (one small long-plan extraction per
arithmetic form on cuda:0, compared with the oracle), run as a GPU test."""
import os
import sys

import pytest

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_smoke_entry_point():
    if REPO not in sys.path:
        sys.path.insert(0, REPO)
    import __graft_entry__
    __graft_entry__.smoke()
