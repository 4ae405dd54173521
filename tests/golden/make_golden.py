"""Extract the reference crate's own known-answer vectors into JSON fixtures.

Run with the path of a reference checkout as the only argument:

    python tests/golden/make_golden.py <path-to-reference-checkout>

It parses the test constants of the vendored generator crate and the literal
matrices of the solver/driver tests, so nothing here is typed by hand:

* rust-random123/src/philox.rs:242-292   TEST_VEC_{2X32,2X64,4X32,4X64}
* rust-random123/src/philox.rs:294-295   SEED1 / SEED2 keys
* rust-random123/src/threefry.rs:97-110  TEST_VEC_1, SEED1_U64, SEED2_U64
* src/solvers.rs:290-338                 upper-triangular solve cases
* src/solvers.rs:391-410                 lsqr 3x2 system, x ~ [1, -1]
* src/cg.rs:130-184                      cgls 3x3 cases
* src/lora_drivers.rs:506-514, 702-710   the 3 x 3 matrix rand_evd1 / rand_evd2 reject

The fixtures are committed; the tests read only the JSON, never the
reference tree.
"""
import json
import os
import re
import sys


def _array(text, name):
    m = re.search(r"const\s+%s\s*:\s*\[(u32|u64);\s*(\d+)\]\s*=\s*\[(.*?)\];" % name,
                  text, re.S)
    if not m:
        raise SystemExit("array %s not found" % name)
    vals = [int(tok.strip(), 16) for tok in m.group(3).split(",") if tok.strip()]
    assert len(vals) == int(m.group(2)), name
    return vals


def _const(text, name):
    m = re.search(r"const\s+%s\s*:\s*u(32|64)\s*=\s*(0x[0-9a-fA-F]+)\s*;" % name, text)
    if not m:
        raise SystemExit("const %s not found" % name)
    return int(m.group(2), 16)


def _row_slice(text, start_pat):
    """Return the numbers of the first from_row_slice(...) after start_pat."""
    i = text.index(start_pat)
    m = re.search(r"from_row_slice\((\d+),\s*(\d+),\s*&\[(.*?)\]\)", text[i:], re.S)
    rows, cols = int(m.group(1)), int(m.group(2))
    vals = [float(t) for t in re.findall(r"-?\d+\.\d+|-?\d+", m.group(3))]
    assert len(vals) == rows * cols
    return rows, cols, vals, i + m.end()


def main(ref):
    with open(os.path.join(ref, "rust-random123/src/philox.rs")) as f:
        philox = f.read()
    with open(os.path.join(ref, "rust-random123/src/threefry.rs")) as f:
        threefry = f.read()
    with open(os.path.join(ref, "src/solvers.rs")) as f:
        solvers = f.read()
    with open(os.path.join(ref, "src/cg.rs")) as f:
        cg = f.read()
    with open(os.path.join(ref, "src/lora_drivers.rs")) as f:
        drivers = f.read()

    rng = {
        "source": "rust-random123/src/philox.rs:242-295, threefry.rs:97-110",
        "philox_key_seed1": _const(philox, "SEED1"),
        "philox_key_seed2": _const(philox, "SEED2"),
        "philox2x32": _array(philox, "TEST_VEC_2X32"),
        "philox2x64": _array(philox, "TEST_VEC_2X64"),
        "philox4x32": _array(philox, "TEST_VEC_4X32"),
        "philox4x64": _array(philox, "TEST_VEC_4X64"),
        "threefry2x64": _array(threefry, "TEST_VEC_1"),
        "threefry_key0": _const(threefry, "SEED1_U64"),
        "threefry_key1": _const(threefry, "SEED2_U64"),
        "counters": "ctr = [i, 0, ...] for i in 0..10 (philox.rs:301-363, threefry.rs:114-127)",
    }

    tri = []
    for name in ("fn test_upper_triangular_basic", "fn test_upper_triangular_zero_diagonal"):
        r, c, u, end = _row_slice(solvers, name)
        _, _, y, _ = _row_slice(solvers[end:], "from_row_slice")
        case = {"name": name.split()[-1], "n": r, "u_rowmajor": u, "y": y}
        if "basic" in name:
            i = solvers.index(name)
            m = re.search(r"let expected = DMatrix::from_row_slice\(3, 1, &\[(.*?)\]\)", solvers[i:], re.S)
            case["expected"] = [float(t) for t in m.group(1).split(",")]
        tri.append(case)

    i = solvers.index("fn test_simple_system")
    r, c, a, _ = _row_slice(solvers, "fn test_simple_system")
    m = re.search(r"let b = dvector!\[(.*?)\];\s*let \(x, istop.*?let b = dvector!\[(.*?)\];",
                  solvers[i:], re.S)
    lsqr_case = {
        "source": "src/solvers.rs:391-410",
        "m": r, "n": c, "a_rowmajor": a,
        "b_zero": [float(t) for t in m.group(1).split(",")],
        "b_known": [float(t) for t in m.group(2).split(",")],
        "x_known": [1.0, -1.0], "abs_tol": 1e-2,
        "damp": 0.0, "atol": 1e-8, "btol": 1e-8, "conlim": 1e8,
    }

    cg_cases = []
    for name in ("fn test_cgls_converges", "fn test_cgls_with_initial_guess",
                 "fn test_cgls_does_not_converge"):
        r, c, a, end = _row_slice(cg, name)
        _, _, b, end2 = _row_slice(cg[end:], "from_row_slice")
        j = cg.index(name)
        body = cg[j:j + 1200]
        tol = float(re.search(r"let tolerance = ([0-9.e-]+);", body).group(1))
        iters = int(re.search(r"let num_iterations = (\d+);", body).group(1))
        x0 = None
        if "initial_guess" in name:
            _, _, x0, _ = _row_slice(cg[end + end2:], "from_row_slice")
        cg_cases.append({"name": name.split()[-1], "a_rowmajor": a, "b": b,
                         "tolerance": tol, "num_iterations": iters, "x0": x0})

    # the non-symmetric matrix both rand_evd drivers must reject
    evd = {}
    for name in ("fn test_wrong_hermitian", "fn test_wrong_psd"):
        j = drivers.index(name)
        m = re.search(r"dmatrix!\[(.*?)\];", drivers[j:], re.S)
        rows = [[float(t) for t in row.split(",")] for row in m.group(1).split(";")]
        evd[name.split()[-1]] = rows

    solv = {"source": "src/solvers.rs, src/cg.rs, src/lora_drivers.rs", "upper_triangular": tri,
            "lsqr_simple": lsqr_case, "cgls": cg_cases, "rand_evd_reject": evd}

    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "rng_kat.json"), "w") as f:
        json.dump(rng, f, indent=1)
    with open(os.path.join(here, "solver_kat.json"), "w") as f:
        json.dump(solv, f, indent=1)
    print("wrote rng_kat.json, solver_kat.json")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path-to-reference-checkout>")
    main(sys.argv[1])
