"""The legacy entry points keep the reference's error behaviour (message
and exit(1)) for calls it rejects before any evaluation; runs without a
GPU (each case in a child process)."""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

SNIPPET = """
import sys
sys.path.insert(0, {pkg!r})
sys.path.insert(0, {tests!r})
import legacy_helpers as L
lib = L.load()
{call}
print("returned")
"""


def run(call):
    code = SNIPPET.format(pkg=os.path.join(ROOT, "cocoa-cosmolike-core_gb300"), tests=HERE, call=call)
    return subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)


def test_nonlimber_xi_exits():
    r = run("lib.xi_pm_tomo(1, 0, 0, 0, 0)")
    assert r.returncode == 1, (r.returncode, r.stdout, r.stderr)
    assert "NonLimber not implemented" in r.stderr
    assert "returned" not in r.stdout


def test_query_before_state_exits():
    r = run("lib.C_gg_tomo_limber(100.0, 0, 0)")
    assert r.returncode == 1, (r.returncode, r.stdout, r.stderr)
    assert "not set" in r.stderr
