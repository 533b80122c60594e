"""The entry point's smoke check (one small diffusion job in the FP64 form
against the oracle) runs as a test too."""
import os
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_smoke(nudim_built):
    sys.path.insert(0, ROOT)
    import __graft_entry__
    __graft_entry__.smoke()
