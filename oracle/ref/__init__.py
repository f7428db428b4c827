"""Builds and launchers of the reference's own code (test infrastructure)."""
from __future__ import annotations

import os
from pathlib import Path

_RECORD = Path(__file__).resolve().parent.parent / "_ref" / "reference_dir.txt"


def reference_dir() -> Path | None:
    """Directory of the reference sources: $NUFI_REFERENCE_DIR, else the one
    oracle/ref/Makefile was last run with (recorded in oracle/_ref/), else
    None (the sources are absent, as on machines without them)."""
    env = os.environ.get("NUFI_REFERENCE_DIR")
    if env:
        return Path(env)
    try:
        d = Path(_RECORD.read_text().strip())
    except OSError:
        return None
    return d if d.is_dir() else None
