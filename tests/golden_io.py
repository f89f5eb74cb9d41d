"""Loader for the committed golden fixtures (tests/golden/*.npz)."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

from common import Case

GOLDEN = Path(__file__).resolve().parent / "golden"


def load(name):
    z = np.load(GOLDEN / f"{name}.npz")
    spec = json.loads(bytes(z["spec"]).decode())
    out = []
    for s in spec:
        args = [z[a["array"]].copy() if isinstance(a, dict) else a for a in s["args"]]
        case = Case(s["op"], args, [int(k) for k in s["outputs"]], scalar=s["scalar"], nred=s["nred"],
                    exact=s["exact"], label=s["label"])
        expected = {int(k): z[v] for k, v in s["outputs"].items()}
        out.append((case, s["result"], expected))
    return out


def names():
    return sorted(p.stem for p in GOLDEN.glob("*.npz"))
