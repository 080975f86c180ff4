"""Input-file front end: run or check a MaCaw-style input (HIT blocks).

The parsing, object construction and parameter checks are in C++
(csrc/mc_app.cpp, exported as mc_app_run / mc_app_check); this module only
passes the text through and decodes the JSON report.
"""
from __future__ import annotations

import ctypes as C
import json
from pathlib import Path

from ._lib import lib

INPUTS = Path(__file__).resolve().parent / "inputs"


def _call(fn, *args) -> tuple[int, dict]:
    buf = C.create_string_buffer(1 << 16)
    rc = fn(*args, buf, len(buf))
    return rc, json.loads(buf.value.decode() or "{}")


def check_input(text: str) -> dict:
    """Parse and validate without a GPU; raises ValueError with the object/parameter path."""
    rc, rep = _call(lib.mc_app_check, text.encode())
    if rc != 0:
        raise ValueError(rep.get("error", f"mc_app_check failed ({rc})"))
    return rep


def run_input(text: str, device: int = 0, file_base: str | None = None) -> dict:
    """Run every batch of the input on the GPU; returns the JSON summary."""
    rc, rep = _call(lib.mc_app_run, text.encode(), device, (file_base or "").encode())
    if rc != 0:
        raise RuntimeError(rep.get("error", f"mc_app_run failed ({rc})"))
    return rep


def read(name: str) -> str:
    return (INPUTS / name).read_text()


def main(argv: list[str] | None = None) -> int:
    """python -m macaw_gb300.app INPUT [--check] [--file-base BASE]: run (or
    only check) an input file and print its JSON report."""
    import argparse
    ap = argparse.ArgumentParser(prog="python -m macaw_gb300.app")
    ap.add_argument("input")
    ap.add_argument("--check", action="store_true", help="parse and validate only (no GPU)")
    ap.add_argument("--file-base", default=None, help="output file base (CSV, Exodus)")
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args(argv)
    text = Path(args.input).read_text()
    rep = check_input(text) if args.check else run_input(text, args.device, args.file_base)
    print(json.dumps(rep, indent=1))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
