"""The C++ plugin path: a user launcher registered in sim::Simulator's
KernelDispatcher (PhaseType::Post) replaces the built-in phase.

tests/cpp/plugin_path.cu is compiled by __graft_entry__.build() against
include/pbf/simulator.h and libpbf_gb300.so (the C++ half of the boundary,
which the ctypes tests do not reach).  It checks that its launcher ran once
(at graph capture), that the scene stepped with it equals the built-in step
of the same scene with XSPH off (its launcher commits without XSPH), and that
the built-in step with XSPH on differs.
"""
import os
import subprocess

import pytest


def test_plugin_program_is_built(built):
    import __graft_entry__ as g

    assert os.path.exists(g.build_plugin_test())


@pytest.mark.gpu
def test_user_post_launcher_replaces_the_built_in_phase(gpu, built):
    import __graft_entry__ as g

    exe = g.build_plugin_test()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "PLUGIN OK calls=1" in r.stdout
