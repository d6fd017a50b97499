"""Build the CUDA extension ``libvajax_gb300.so`` for sm_103a.

Steps: emit the CUDA source of every bundled device model from its committed
MIR fixture (``devices/*.json``), compile each translation unit with nvcc in
parallel, and link one shared library next to this file.  The library is a
plain C ABI (``include/vajax_gb300.h``); Python reaches it through ctypes.
"""

from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libvajax_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["vgb_api.cu", "vgb_transient.cu", "vgb_kernels.cu", "vgb_frontal.cu", "vgb_dense_static.cu",
           "vgb_batch.cu", "vgb_host.cpp"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build vajax_gb300")
    return exe


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(CSRC), "-I", str(BUILD),
                   "-I", str(ROOT / "include"), "--expt-relaxed-constexpr"]


def _compile(src: Path, obj: Path, extra=()):
    cmd = [nvcc(), *(_flags()), *extra, "-c", str(src), "-o", str(obj)]
    if src.suffix == ".cpp":
        cmd = [nvcc(), "-x", "cu", *(_flags()), *extra, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stderr[-4000:]}")
    return obj


def math_tables() -> str:
    """Tables and split constants of the device elementary functions
    (csrc/vgb_math.cuh), from 50-digit decimal arithmetic rounded once to
    double: 2^(j/64) for j = 0..63; 1/F, ln F (as a head and a tail) for
    F = 1 + j/128, j = 0..128; ln2/64 and ln2 split into a head with few
    enough significant bits that its products with the reduction integers
    are exact, and a tail."""
    import decimal
    import struct
    D = decimal.Decimal
    decimal.getcontext().prec = 50
    ln2 = D(2).ln()

    def head(x: D, bits: int) -> float:
        v = struct.unpack("<Q", struct.pack("<d", float(x)))[0]
        return struct.unpack("<d", struct.pack("<Q", v & ~((1 << (52 - bits + 1)) - 1)))[0]

    def arr(name, vals):
        body = ",\n    ".join(float(v).hex() for v in vals)
        return f"static __device__ const double {name}[{len(vals)}] = {{\n    {body}}};"

    ln2_64 = ln2 / 64
    ln2_64_hi = head(ln2_64, 36)
    ln2_hi = head(ln2, 42)
    exp2 = [float((D(j) / 64 * ln2).exp()) for j in range(64)]
    inv_f, lnf_hi, lnf_lo = [], [], []
    for j in range(129):
        F = 1 + D(j) / 128
        inv_f.append(float(1 / F))
        lnf = F.ln()
        hi = ln2_hi if j == 128 else float(lnf)
        lnf_hi.append(hi)
        lnf_lo.append(float(lnf - D(hi)))
    consts = {
        "VGB_INV_LN2_64": float(64 / ln2), "VGB_LN2_64_HI": ln2_64_hi, "VGB_LN2_64_LO": float(ln2_64 - D(ln2_64_hi)),
        "VGB_LN2_HI": ln2_hi, "VGB_LN2_LO": float(ln2 - D(ln2_hi)), "VGB_INV_LN10": float(1 / D(10).ln()),
    }
    lines = ["// Generated by vajax_gb300/build.py (math_tables); do not edit.", "#pragma once"]
    lines += [f"#define {k} ({v.hex()})" for k, v in consts.items()]
    lines += [arr("VGB_EXP2_TAB", exp2), arr("VGB_LOG_INVF", inv_f), arr("VGB_LOG_LNF_HI", lnf_hi),
              arr("VGB_LOG_LNF_LO", lnf_lo)]
    return "\n".join(lines) + "\n"


def _write_if_changed(path: Path, text: str):
    if not path.exists() or path.read_text() != text:
        path.write_text(text)


def generate_models() -> Path:
    sys.path.insert(0, str(ROOT))
    from vajax_gb300.codegen.cuda import write_generated
    BUILD.mkdir(exist_ok=True)
    out = BUILD / "vgb_models_gen.cu"
    tmp = BUILD / "vgb_models_gen.cu.tmp"
    _write_if_changed(BUILD / "vgb_math_tables.cuh", math_tables())
    write_generated(PKG / "devices", tmp, BUILD / "vgb_models_gen.cuh")
    if not out.exists() or out.read_bytes() != tmp.read_bytes():
        tmp.replace(out)
    else:
        tmp.unlink()
    return out


def _digest(paths) -> str:
    h = hashlib.sha256()
    for p in paths:
        h.update(p.name.encode())
        h.update(p.read_bytes())
    h.update(" ".join(_flags()).encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> Path:
    gen = generate_models()
    srcs = [CSRC / s for s in SOURCES] + [gen]
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + [ROOT / "include" / "vajax_gb300.h",
                                                                        BUILD / "vgb_math_tables.cuh",
                                                                        BUILD / "vgb_models_gen.cuh"]
    digest = _digest(srcs + headers)
    stamp = BUILD / "stamp"
    if not force and LIB.exists() and stamp.exists() and stamp.read_text() == digest:
        return LIB
    BUILD.mkdir(exist_ok=True)
    objs = []
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        futs = []
        for s in srcs:
            obj = BUILD / (s.stem + ".o")
            extra = ["-Xptxas", "-v"] if verbose else []
            futs.append(ex.submit(_compile, s, obj, extra))
        for f in futs:
            objs.append(f.result())
    tmp_lib = BUILD / "libvajax_gb300.so.tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp_lib), *map(str, objs)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    tmp_lib.replace(LIB)
    stamp.write_text(digest)
    return LIB


if __name__ == "__main__":
    import time
    t = time.time()
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv), f"{time.time() - t:.1f}s")
