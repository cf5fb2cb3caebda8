"""GPU: the bounds-checked debug build (RT_CHECKS; compute-sanitizer is not
available) renders every layout with no index out of bounds and the same
images as the normal build, bit for bit.

Every node, record, instance and thing index that traversal and shading read
from memory is checked in that build; a bad one would set an error bit and
fail the call with RT_ERR_INTERNAL.  The checked library runs in a child
process (RTX_LIB) so that the two builds never share a process.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_checked_build_renders_identically(product, cuda, tmp_path):
    from rtxplay_gb300 import _build
    sys.path.insert(0, HERE)
    import _checked_run
    checked = _build.build_checked()
    ref = str(tmp_path / "ref.npz")
    np.savez(ref, **_checked_run.renders())
    env = dict(os.environ, RTX_LIB=checked, PYTHONPATH=os.pathsep.join([os.path.dirname(HERE), HERE]))
    r = subprocess.run([sys.executable, os.path.join(HERE, "_checked_run.py"), ref], env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0 and "checked ok" in r.stdout, r.stdout + r.stderr
