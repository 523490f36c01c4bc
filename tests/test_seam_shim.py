"""The narrow seam's reference-side backend (calcqpi-release_gb300/seam/gb300qpi.h): compiled
against the reference's own GPUQPI interface and linked with libcqpi.so by oracle/build_ref.sh
(oracle/_ref/seam_check, present where the reference sources were available to build it).
CPU only: the check proves the backend compiles and links, and that an engine error (here: no
usable GPU) reaches the reference's code as an exception."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CHECK = os.path.join(ROOT, "oracle", "_ref", "seam_check")


@pytest.fixture(scope="module")
def seam_check(built_lib):
    if not os.path.exists(CHECK):
        pytest.skip("oracle/_ref/seam_check not built (the reference sources are needed)")
    return CHECK


def test_backend_links_against_reference_interface(seam_check):
    r = subprocess.run([seam_check], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip().endswith("linked")


def test_backend_reports_engine_errors_as_exceptions(seam_check):
    r = subprocess.run([seam_check, "create"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert ("threw: GB300QPI: cqpi_create" in r.stdout) or ("created" in r.stdout)
