"""The smoke check run before the benchmark: one step of a 512-particle scene
in both grid modes against the oracle, with the step tests' parity bars."""
import os
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_smoke(gpu):
    sys.path.insert(0, ROOT)
    import __graft_entry__ as g

    g.smoke()
