"""Loads the golden fixtures (tests/golden/*.json) and maps their problems to the oracle's
and the engine's parameter types."""
from __future__ import annotations

import json
import os

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    with open(os.path.join(HERE, name)) as f:
        return json.load(f)


def cases(kind=None):
    data = load("reference_cases.json")["cases"]
    return [c for c in data if kind is None or c["kind"] == kind]


def codes(texts, alphabet):
    from seqan_gb300.alphabet import encode
    return [encode(t, "aa" if alphabet == "aa" else "dna5") for t in texts]


def oracle_problem(p):
    from oracle.oracle import Problem
    mat = np.array(load("blosum62.json")["matrix"], dtype=np.int32) if p["blosum62"] else None
    return Problem(p["mode"], p["free_ends"], tuple(p["band"]) if p["band"] else None, p["match"],
                   p["mismatch"], p["gap_open"], p["gap_extend"], mat, p["score_bits"], p["alphabet"])


def engine_args(p):
    """(score, mode, AlignConfig, band) for seqan_gb300.align_codes."""
    import seqan_gb300 as sg
    dtype = np.int16 if p["score_bits"] == 16 else np.int32
    if p["blosum62"]:
        score = sg.Blosum62(p["gap_extend"], p["gap_open"], dtype=dtype)
    else:
        score = sg.Score(p["match"], p["mismatch"], p["gap_extend"], p["gap_open"], dtype=dtype)
    fe = p["free_ends"]
    cfg = sg.AlignConfig(bool(fe & 1), bool(fe & 2), bool(fe & 4), bool(fe & 8))
    mode = 1 if p["mode"] == "local" else 0
    band = tuple(p["band"]) if p["band"] else None
    return score, mode, cfg, band


def case_id(c):
    p = c["problem"]
    return (f"{c['kind']}-{p['mode']}-fe{p['free_ends']}-{p['alphabet']}{p['score_bits']}-"
            f"{p['match']},{p['mismatch']},{p['gap_open']},{p['gap_extend']}" + ("-band" if p["band"] else ""))
