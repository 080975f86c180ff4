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
