"""Raw-file and CSV writers round trip (vajax/io/rawfile_writer.py formats)."""

import numpy as np
import pytest

from vajax_gb300.engine import TransientResult
from vajax_gb300.io import read_rawfile, write_csv, write_rawfile


def _result():
    t = np.linspace(0, 1e-9, 11)
    return TransientResult(times=t, voltages={"out": np.sin(t * 1e9), "in": np.cos(t * 1e9)}, currents={}, stats={})


@pytest.mark.parametrize("binary", [True, False])
def test_rawfile_round_trip(tmp_path, binary):
    r = _result()
    p = tmp_path / "x.raw"
    write_rawfile(r, p, binary=binary)
    xname, cols = read_rawfile(p)
    assert xname == "time"
    np.testing.assert_array_equal(cols["time"], r.times)
    np.testing.assert_array_equal(cols["v(out)"], r.voltages["out"])
    np.testing.assert_array_equal(cols["v(in)"], r.voltages["in"])
    head = p.read_bytes().split(b"Binary:" if binary else b"Values:")[0].decode()
    assert "No. Variables: 3" in head and "No. Points: 11" in head and "Plotname: Transient Analysis" in head


def test_csv(tmp_path):
    r = _result()
    p = tmp_path / "x.csv"
    write_csv(r, p)
    data = np.loadtxt(p, delimiter=",", skiprows=1)
    np.testing.assert_array_equal(data[:, 0], r.times)
    np.testing.assert_array_equal(data[:, 2], r.voltages["in"])
