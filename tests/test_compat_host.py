"""Host-side logic of the package-facing compatibility layer (task lists, input deck,
parameters, metadata, integrator tables, sparse pools, pack index lookups, reducers,
package and application hooks), built with nvcc and run on the CPU."""
import os
import subprocess

from compat_build import ROOT, compile_objects, link


def test_compat_host_logic():
    objs = compile_objects([os.path.join(ROOT, "tests", "cxx", "compat_host_check.cpp")], "compathost")
    exe = link(objs, "compat_host_check")
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr
