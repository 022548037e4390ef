"""The drop-in command line (lulesh_gb300/bin/lulesh_gpu) against the
reference executable's option handling (lulesh-util.cc:63-171): the same
messages and exit codes for help and for every malformed option.  None of
these reach the device, so they run without a GPU."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "lulesh_gb300", "bin", "lulesh_gpu")
REF = os.path.join(ROOT, "oracle", "_ref", "lulesh_ref")

CASES = [["-h"], ["-s"], ["-s", "abc"], ["-i"], ["-i", "5x"], ["-r"], ["-b", ""], ["-c"],
         ["-f"], ["-v"], ["-x"], ["-s", "8", "-q", "-b"], ["--bogus"]]


def _run(exe, args):
    r = subprocess.run([exe] + args, capture_output=True, text=True, timeout=60)
    return r.returncode, r.stdout + r.stderr


def _normalise(text, exe):
    # the executable's own name, and the device options only this CLI has
    text = text.replace(exe, "EXE")
    return "\n".join(l for l in text.splitlines()
                     if not re.match(r"^ --(precision|device|viz-vtk)\b", l))


@pytest.fixture(scope="module")
def cli(native_lib):
    assert os.path.exists(CLI)
    return CLI


@pytest.mark.parametrize("args", CASES, ids=[" ".join(a) or "empty" for a in CASES])
def test_option_handling_matches_reference(cli, args):
    if not os.path.exists(REF):
        pytest.skip("reference executable not built here")
    rc_ref, out_ref = _run(REF, args)
    rc, out = _run(cli, args)
    assert rc == rc_ref
    assert _normalise(out, cli) == _normalise(out_ref, REF)


def test_viz_needs_the_reference_build_flag(cli):
    rc, out = _run(cli, ["-v"])
    assert rc == 255 and "Use of -v requires compiling with -DVIZ_MESH" in out
    rc, out = _run(cli, ["--viz-vtk"])
    assert rc == 255 and "Missing argument to --viz-vtk" in out
