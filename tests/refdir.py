"""Where tests look for a checkout of the reference project (BayesRRcmd).

The checkout is optional: tests that read its fixtures or sources skip when
it is absent.  BRR_REFERENCE_DIR names it; without the variable a checkout
named `reference` beside this repository is used when one exists.
"""
import os
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def reference_dir() -> Path:
    env = os.environ.get("BRR_REFERENCE_DIR")
    return Path(env) if env else ROOT.parent / "reference"
