"""The ncu instruction counts the bench's rooflines read (profiles/*_counts.json)
must describe the kernels as they are: each file records the SHA-256 of the
kernel's sources at capture time, and the bench prints null counts when they
differ.  This check fails first, on the CPU, so that an edit to a counted kernel
is followed by a new capture (the command is in each file)."""
import json
import os

import pytest

from conftest import REPO

COUNTS = ["direct_kernel_counts.json", "tree_walk_counts.json", "ensemble_kernel_counts.json"]


def digest(paths):
    import hashlib
    h = hashlib.sha256()
    for rel in paths:
        with open(os.path.join(REPO, rel), "rb") as f:
            h.update(f.read())
    return h.hexdigest()


@pytest.mark.parametrize("name", COUNTS)
def test_counts_match_kernel_sources(name):
    with open(os.path.join(REPO, "profiles", name)) as f:
        rec = json.load(f)
    assert rec["sources"] and rec["ncu_command"].startswith("ncu --clock-control none")
    assert digest(rec["sources"]) == rec["sha256"], (
        f"{name}: the kernel sources changed since the ncu capture; recapture with: {rec['ncu_command']}")


def test_bench_reads_the_same_digest():
    import sys
    sys.path.insert(0, REPO)
    import bench
    for name in COUNTS:
        with open(os.path.join(REPO, "profiles", name)) as f:
            rec = json.load(f)
        assert bench.sources_digest(rec["sources"]) == digest(rec["sources"])
