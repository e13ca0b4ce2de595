"""The .osh restatement used as the checker (tests/osh_format.py) against
files the reference itself wrote: it reads them to the reference's own mesh
arrays, and writing what it read gives the same bytes."""
import filecmp
import os

import numpy as np
import pytest

import osh_format as osh

HERE = os.path.dirname(os.path.abspath(__file__))
OSH = os.path.join(HERE, "golden", "osh")
CASES = sorted(os.listdir(OSH))


@pytest.mark.parametrize("case", CASES)
def test_reads_the_reference_arrays(case):
    m = osh.read(os.path.join(OSH, case, "out.osh"))
    want = dict(np.load(os.path.join(OSH, case, "out_arrays.npz")))
    dim = m["dim"]
    assert m["nverts"] == want["out_coords"].size // dim
    for d in range(1, dim + 1):
        assert np.array_equal(m["down"][d], want[f"out_down_{d}"])
        if d > 1:
            assert np.array_equal(m["codes"][d], want[f"out_downcodes_{d}"])
    assert np.array_equal(osh.tag(m, 0, "coordinates"), want["out_coords"])
    assert np.array_equal(osh.tag(m, 0, "metric"), want["out_metric"])
    for d in range(dim + 1):
        assert np.array_equal(osh.tag(m, d, "global"), np.arange(m["tags"][d][0][3].size))
        assert np.array_equal(osh.tag(m, d, "class_id"), want[f"out_class_id_{d}"])
        assert np.array_equal(osh.tag(m, d, "class_dim"), want[f"out_class_dim_{d}"])
    assert np.array_equal(osh.tag(m, 1, "length"), want["out_length"])
    assert np.array_equal(osh.tag(m, dim, "quality"), want["out_quality"])


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("part", ["in.osh", "out.osh"])
def test_write_of_read_is_byte_identical(tmp_path, case, part):
    src = os.path.join(OSH, case, part)
    osh.write(str(tmp_path / "x.osh"), osh.read(src))
    for f in ("0.osh", "nparts", "version"):
        assert filecmp.cmp(os.path.join(src, f), str(tmp_path / "x.osh" / f), shallow=False), f


def test_compressed_round_trip(tmp_path):
    m = osh.read(os.path.join(OSH, CASES[0], "out.osh"))
    m["compressed"] = 1
    osh.write(str(tmp_path / "z.osh"), m)
    z = osh.read(str(tmp_path / "z.osh"))
    assert z["compressed"] == 1 and not osh.compare(m, z, rtol=0.0)
