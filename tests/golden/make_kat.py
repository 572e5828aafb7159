"""Extract BOLA's own known-answer tests into tests/golden/bola_kat.json.

Reads the Rust test sources of the BOLA crate (the crate's root directory,
a required argument) as TEXT: each listed test function's `let` literals
(arrays and scalars) are parsed out, and the call it makes is recorded with
the file:line of the test.  The JSON it writes is the fixture the test-suite
uses; the suite itself never reads the BOLA sources.

    python tests/golden/make_kat.py <path-to-bola-crate>
"""
import json
import os
import re
import sys

if len(sys.argv) != 2:
    sys.exit("usage: make_kat.py <path-to-bola-crate>")
ROOT = sys.argv[1]
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "bola_kat.json")

# (file, test fn, routine, call arguments in BOLA's order; names refer to the
#  test's `let` bindings, literals are written as-is in the Rust call)
CASES = [
    ("src/gemm.rs", "test_gemm_matrix_multiplication", "gemm",
     ["'N'", "'N'", "m", "n", "k", 1.0, "a", "lda", "b", "ldb", 0.0, "c", "ldc"], "c", "c_expected", 1e-8),
    ("src/gemm.rs", "test_gemm_n_n", "gemm",
     ["'N'", "'N'", "m", "n", "k", 1.0, "a", "lda", "b", "ldb", 0.0, "c", "ldc"], "c", "c_expected", 1e-9),
    ("src/gemm.rs", "test_gemm_n_t", "gemm",
     ["'N'", "'T'", "m", "n", "k", 1.0, "a", "lda", "b", "ldb", 0.0, "c", "ldc"], "c", "c_expected", 1e-9),
    ("src/laswp.rs", "test_laswp_row_swaps", "laswp",
     ["n_cols_to_swap", "a", "lda", 1, 2, "ipiv", 1], "a", "a_expected", 1e-8),
    ("src/scal.rs", "test_scal_kernel_logic", "scal", ["#len(x)", "a", "x", 1], "x", "expected", 0.0),
    ("src/syrk.rs", "test_syrk_lower_no_transpose", "syrk",
     ["'L'", "'N'", "n", "k", 1.0, "a", "lda", 1.0, "c", "ldc"], "c", "c_expected", 1e-9),
    ("src/syrk.rs", "test_syrk_upper_transpose", "syrk",
     ["'U'", "'T'", "n", "k", 1.0, "a", "lda", 1.0, "c", "ldc"], "c", "c_expected", 1e-9),
    ("src/trsm.rs", "test_trsm_left_lower_no_transpose", "trsm",
     ["'L'", "'L'", "'N'", "'N'", "m", "n", 1.0, "a", "lda", "b", "ldb"], "b", "x_expected", 1e-9),
    ("src/trsm.rs", "test_trsm_right_upper_transpose", "trsm",
     ["'R'", "'U'", "'T'", "'N'", "m", "n", 1.0, "a", "lda", "b", "ldb"], "b", "x_expected", 1e-9),
    ("src/trsm.rs", "test_trsm_right_lower_transpose", "trsm",
     ["'R'", "'L'", "'T'", "'N'", "m", "n", 1.0, "a", "lda", "b", "ldb"], "b", "x_expected", 1e-9),
    ("tests/integration.rs", "test_potrf_cholesky_factorisation_upper", "potrf",
     ["'U'", "n", "a", "lda"], "a", "u_expected", 1e-9),
    ("tests/integration.rs", "test_potrf_cholesky_factorisation_lower", "potrf",
     ["'L'", "n", "a", "lda"], "a", "l_expected", 1e-9),
    ("tests/integration.rs", "test_getrf_lu_decomposition", "getrf",
     ["m", "n", "a", "lda", "ipiv"], "a", "lu_expected", 1e-4),
]

ARR = re.compile(r"let\s+(?:mut\s+)?(\w+)\s*(?::[^=]+)?=\s*(?:vec!)?\[([^\]]*)\]\s*;")
SCA = re.compile(r"let\s+(?:mut\s+)?(\w+)\s*=\s*(-?[0-9][0-9_.eE+-]*)\s*;")
FILL = re.compile(r"let\s+(?:mut\s+)?(\w+)\s*=\s*(?:vec!)?\[\s*(-?[0-9.]+)\s*;\s*(\w+|[0-9]+)\s*\]\s*;")


def num(tok):
    tok = tok.strip().replace("_", "")
    return float(tok) if any(ch in tok for ch in ".eE") else int(tok)


def body_of(text, fn):
    start = text.index("fn " + fn + "(")
    nxt = text.find("#[test]", start)
    return start, text[start: nxt if nxt > 0 else len(text)]


def main():
    cases = []
    for path, fn, routine, args, out_name, exp_name, tol in CASES:
        text = open(os.path.join(ROOT, path)).read()
        start, body = body_of(text, fn)
        line = text[:start].count("\n") + 1
        env = {}
        for name, val in SCA.findall(body):
            env[name] = num(val)
        for name, val, cnt in FILL.findall(body):
            count = env[cnt] if cnt in env else int(cnt)
            env[name] = [num(val)] * count
        for name, items in ARR.findall(body):
            if ";" in items:
                continue  # `[value; count]` fills are handled above
            env[name] = [num(t) for t in items.split(",") if t.strip()]
        # `vec![0; 3]` style fills whose count is an expression (n * n)
        for name, val, expr in re.findall(r"let\s+(?:mut\s+)?(\w+)\s*=\s*vec!\[\s*([0-9.]+)\s*;\s*([\w\s*]+)\]", body):
            if name not in env:
                count = eval(expr, {}, dict(env))
                env[name] = [num(val)] * count
        resolved = []
        for a in args:
            if isinstance(a, str) and a.startswith("'"):
                resolved.append(a.strip("'"))
            elif isinstance(a, str) and a.startswith("#len("):
                resolved.append(len(env[a[5:-1]]))
            elif isinstance(a, str):
                resolved.append(env[a])
            else:
                resolved.append(a)
        case = {
            "source": f"{path}:{line}", "test": fn, "routine": routine, "args": resolved,
            "output_arg": args.index(out_name), "expected": env[exp_name], "tol": tol,
        }
        if routine == "getrf":
            case["expected_ipiv"] = env["ipiv_expected"]
        if routine in ("syrk", "potrf"):
            case["compare_triangle"] = True
        cases.append(case)
    with open(OUT, "w") as f:
        json.dump({"generator": "tests/golden/make_kat.py", "cases": cases}, f, indent=1)
    print(f"wrote {len(cases)} cases to {OUT}")


if __name__ == "__main__":
    main()
