"""Result writers: SPICE raw files (ASCII or binary) and CSV.

The raw format is the one ngspice's ``write`` produces and ``rawread`` /
waveform viewers read: a text header (title, date, plot name, flags, variable
and point counts, the variable table) followed by ``Values:`` in text or
``Binary:`` with one little-endian float64 per variable per point, point-major.
Same entry points as the reference's writers (``vajax/io/rawfile_writer.py``
``write_rawfile``; ``vajax/io/csv_writer.py``); ``read_rawfile`` reads both
forms back.
"""

from __future__ import annotations

import datetime
from pathlib import Path
from typing import Dict, Tuple, Union

import numpy as np


def _columns(result) -> Tuple[str, np.ndarray, Dict[str, np.ndarray]]:
    if hasattr(result, "frequencies"):
        return "frequency", np.asarray(result.frequencies), {k: np.asarray(v) for k, v in result.voltages.items()}
    return "time", np.asarray(result.times, np.float64), {k: np.asarray(v, np.float64)
                                                         for k, v in result.voltages.items()}


def _header(title: str, plot: str, xname: str, names, n_points: int) -> str:
    lines = [f"Title: {title}", f"Date: {datetime.datetime.now().strftime('%a %b %d %H:%M:%S %Y')}",
             f"Plotname: {plot}", "Flags: real", f"No. Variables: {len(names) + 1}", f"No. Points: {n_points}",
             "Variables:", f"\t0\t{xname}\t{xname}"]
    lines += [f"\t{i}\tv({n})\tvoltage" for i, n in enumerate(names, start=1)]
    return "\n".join(lines) + "\n"


def write_rawfile(result, output_path: Union[str, Path], binary: bool = True, title: str = "vajax-gb300") -> None:
    xname, x, volts = _columns(result)
    names = list(volts)
    plot = "AC Analysis" if xname == "frequency" else "Transient Analysis"
    data = np.column_stack([x] + [volts[n] for n in names]) if names else x[:, None]
    head = _header(title, plot, xname, names, len(x))
    path = Path(output_path)
    if binary:
        with open(path, "wb") as fh:
            fh.write(head.encode("ascii"))
            fh.write(b"Binary:\n")
            fh.write(np.ascontiguousarray(data, "<f8").tobytes())
    else:
        with open(path, "w") as fh:
            fh.write(head)
            fh.write("Values:\n")
            for k, row in enumerate(data):
                fh.write(f" {k}\t{row[0]:.17e}\n")
                for v in row[1:]:
                    fh.write(f"\t{v:.17e}\n")


def read_rawfile(path: Union[str, Path]) -> Tuple[str, Dict[str, np.ndarray]]:
    """(x variable name, {name: array}) of a raw file written by write_rawfile."""
    raw = Path(path).read_bytes()
    key = b"Binary:\n" if b"Binary:\n" in raw else b"Values:\n"
    head, body = raw.split(key, 1)
    lines = head.decode("ascii").splitlines()
    nvar = int(next(ln for ln in lines if ln.startswith("No. Variables:")).split(":")[1])
    npts = int(next(ln for ln in lines if ln.startswith("No. Points:")).split(":")[1])
    vi = lines.index("Variables:")
    names = [lines[vi + 1 + i].split("\t")[2] for i in range(nvar)]
    if key == b"Binary:\n":
        data = np.frombuffer(body[: 8 * nvar * npts], "<f8").reshape(npts, nvar)
    else:
        vals = []
        for ln in body.decode("ascii").splitlines():
            parts = ln.split()
            if parts:
                vals.append(float(parts[-1]))
        data = np.asarray(vals).reshape(npts, nvar)
    return names[0], {n: data[:, i].copy() for i, n in enumerate(names)}


def write_csv(result, output_path: Union[str, Path]) -> None:
    xname, x, volts = _columns(result)
    names = list(volts)
    with open(output_path, "w") as fh:
        fh.write(",".join([xname] + [f"v({n})" for n in names]) + "\n")
        for k in range(len(x)):
            fh.write(",".join(f"{v:.17g}" for v in [x[k]] + [volts[n][k] for n in names]) + "\n")
