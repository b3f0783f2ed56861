"""The bounds-checked build (librd_mpm_checked.so, -DRD_BOUNDS_CHECK): every
index the fused kernel and the P2G compute into their shared tiles, records,
particle and grid buffers is tested before the access.  Built here and run in a
child process over the workloads of tests/bounds_check_run.py (edge cases,
batches, FP64, stage mode, the sorted upload, the adjoint): no access may
leave its buffer, and the results stay those of the normal build's checks."""
import json
import os
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_normal_build_reports_unchecked(built_pkg):
    """No GPU needed: the normal build answers without touching the device."""
    if built_pkg.CHECKED:
        pytest.skip("this process loads the checked build")
    assert built_pkg.bounds_violations() == (0, False)


@pytest.mark.gpu
def test_checked_build_finds_no_access_out_of_range(built_pkg):
    env = dict(os.environ, RD_BOUNDS_CHECK="1")
    r = subprocess.run([sys.executable, os.path.join(HERE, "bounds_check_run.py")], env=env, capture_output=True,
                       text=True, timeout=1200)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert res["checked"] is True
    assert res["violations"] == 0, res
    assert res["oracle_one_step"] < 1e-5, res
    flags = res["flags"]
    for k in ("snowball", "batch", "fp64_track_fp", "sorted_upload", "adjoint"):
        assert flags[k] == 0, (k, flags)
    for k in ("edges_30", "edges_37"):  # the particle outside the domain is flagged, nothing else
        assert flags[k] & built_pkg.FLAG_OUT_OF_DOMAIN and not flags[k] & ~built_pkg.FLAG_OUT_OF_DOMAIN, flags
