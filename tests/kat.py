"""Runs BOLA's own known-answer tests (tests/golden/bola_kat.json, extracted
from the BOLA sources by tests/golden/make_kat.py) through any backend that
exposes BOLA's routine names with numpy column-major arrays."""
import json
import os

import numpy as np

KAT_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bola_kat.json")


def load_cases():
    with open(KAT_PATH) as f:
        return json.load(f)["cases"]


def _prep(args):
    out = []
    for a in args:
        if isinstance(a, list):
            if all(isinstance(v, int) for v in a) and a and not any(isinstance(v, float) for v in a):
                out.append(np.array(a, dtype=np.int32))
            else:
                out.append(np.array(a, dtype=np.float64))
        else:
            out.append(a)
    return out


def run_case(backend, case):
    """Returns (result array, expected array, extra dict)."""
    routine = case["routine"]
    args = _prep(case["args"])
    extra = {}
    if routine == "getrf":
        m, n, a, lda, ipiv = args
        ipiv = np.zeros(len(case["args"][4]), dtype=np.int32)
        info = backend.getrf(m, n, a, lda, ipiv)
        extra = {"info": info, "ipiv": ipiv}
        res = a
    elif routine == "potrf":
        uplo, n, a, lda = args
        extra = {"info": backend.potrf(uplo, n, a, lda)}
        res = a
    else:
        getattr(backend, routine)(*args)
        res = args[case["output_arg"]]
    exp = np.array(case["expected"], dtype=np.float64)
    res = np.array(res, dtype=np.float64).ravel()
    if case.get("compare_triangle"):
        # BOLA's tests compare only the computed triangle (the other is zeroed)
        mask = exp != 0.0
        if routine == "potrf" or routine == "syrk":
            n = int(round(np.sqrt(exp.size)))
            idx = np.arange(exp.size)
            i, j = idx % n, idx // n
            upper = case["args"][0] == "U"
            mask = (i <= j) if upper else (i >= j)
        res = np.where(mask, res, 0.0)
    return res, exp, extra


def check_case(backend, case):
    res, exp, extra = run_case(backend, case)
    tol = case["tol"]
    if tol == 0.0:
        assert np.array_equal(res, exp), (case["source"], res, exp)
    else:
        assert np.all(np.abs(res - exp) < tol), (case["source"], res, exp)
    if "expected_ipiv" in case:
        assert extra["info"] == 0
        assert list(extra["ipiv"]) == case["expected_ipiv"], (extra["ipiv"], case["expected_ipiv"])
    if case["routine"] == "potrf":
        assert extra["info"] == 0
