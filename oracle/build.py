"""Build recipe for the oracle (test infrastructure only).

* ``oracle/_build/libt1m_port.so`` — the C++ restatement in
  ``oracle/port/t1m_port.cpp`` (always built; it is what the tests and the CPU
  baseline call on every machine).
* ``oracle/_ref/libt1m_ref.so`` — the UNMODIFIED reference headers instantiated
  through ``oracle/ref_shim.cpp`` against the BLIS stand-in.  Built only where
  the reference source tree exists (``T1M_REFERENCE_DIR``, default: a
  ``reference`` directory beside this repository's root); it is never
  committed and never needed at run time.

Both use ``-ffp-contract=off`` and explicit ``std::fma`` in the micro-kernel so
x86-64 and aarch64 builds produce the same bits.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
PORT_SRC = HERE / "port" / "t1m_port.cpp"
SHIM_SRC = HERE / "ref_shim.cpp"
STANDIN = HERE / "standin"
PORT_LIB = HERE / "_build" / "libt1m_port.so"
REF_LIB = HERE / "_ref" / "libt1m_ref.so"
# The reference checkout: $T1M_REFERENCE_DIR, else a sibling of the repo root.
REFERENCE_DIR = Path(os.environ.get("T1M_REFERENCE_DIR",
                                    str(HERE.parent.parent / "reference")))

CXXFLAGS = ["-O3", "-fPIC", "-shared", "-ffp-contract=off", "-Wall"]


def _stale(target: Path, *sources: Path) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}")


def build_port(force: bool = False) -> Path:
    PORT_LIB.parent.mkdir(parents=True, exist_ok=True)
    if force or _stale(PORT_LIB, PORT_SRC, STANDIN / "blis.h"):
        tmp = PORT_LIB.with_suffix(".so.tmp")
        _run(["g++", "-std=c++17", *CXXFLAGS, "-pthread", f"-I{STANDIN}",
              str(PORT_SRC), "-o", str(tmp)])
        tmp.replace(PORT_LIB)
    return PORT_LIB


def reference_available() -> bool:
    return (REFERENCE_DIR / "include" / "t1m" / "t1m.h").exists()


def build_ref(force: bool = False) -> Path | None:
    if not reference_available():
        return REF_LIB if REF_LIB.exists() else None
    REF_LIB.parent.mkdir(parents=True, exist_ok=True)
    hdr = REFERENCE_DIR / "include" / "t1m" / "t1m.h"
    if force or _stale(REF_LIB, SHIM_SRC, STANDIN / "blis.h", hdr):
        tmp = REF_LIB.with_suffix(".so.tmp")
        _run(["g++", "-std=c++23", *CXXFLAGS, f"-I{STANDIN}",
              f"-I{REFERENCE_DIR / 'include'}", str(SHIM_SRC), "-o", str(tmp)])
        tmp.replace(REF_LIB)
    return REF_LIB


def build(force: bool = False) -> None:
    build_port(force)
    build_ref(force)


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print(PORT_LIB, REF_LIB if REF_LIB.exists() else "(reference shim not built)")
