"""The C ABI library builds, loads and exports every symbol include/dto.h
declares.  Only host-side utilities are called (no GPU needed)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def L():
    from dual_threshold_optimization_gb300 import build
    build.build()
    from dual_threshold_optimization_gb300 import _lib
    return _lib.lib()


def declared():
    src = open(os.path.join(ROOT, "include", "dto.h")).read()
    return re.findall(r"DTO_API\s+[\w\s\*]+?\b(dto_\w+)\s*\(", src)


def test_header_declarations_are_exported(L):
    names = declared()
    assert len(names) >= 20
    from dual_threshold_optimization_gb300 import _lib
    assert set(names) == set(_lib.EXPORTS), set(names) ^ set(_lib.EXPORTS)
    for n in names:
        assert hasattr(L, n), n


def test_host_utilities(L):
    import numpy as np
    from oracle import oracle as O
    from dual_threshold_optimization_gb300._lib import ptr
    for mr in (0, 1, 5, 100, 101, 1000, 20000, 65535):
        n = L.dto_generate_thresholds(mr, None, 0)
        out = np.zeros(max(n, 1), np.uint32)
        L.dto_generate_thresholds(mr, ptr(out), n)
        assert out[:n].tolist() == O.thresholds(mr).tolist()
    assert L.dto_fdr(200, 150, 50, 1000, 0.8) == O.fdr(200, 150, 50, 1000, 0.8)
    assert L.dto_fdr(10, 10, 0, 100, 0.8) == 0.0
    assert L.dto_status_string(0) == b"ok"
    assert L.dto_version() >= 10000


def test_rank_order_is_the_stable_sort(L):
    # dto_pair_create's order by rank (counting sort for dense ranks, radix
    # sort for sparse ones) equals a stable comparison sort, ties in input order
    import numpy as np
    from dual_threshold_optimization_gb300._lib import ptr
    rng = np.random.default_rng(17)
    cases = [np.zeros(0, np.uint32), np.array([7], np.uint32), np.full(1000, 3, np.uint32)]
    for n in (2, 17, 1000, 20000):
        cases.append(rng.permutation(n).astype(np.uint32) + 1)            # dense, no ties
        cases.append(rng.integers(1, max(2, n // 4), n, dtype=np.uint32))  # dense, many ties
        cases.append(rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32))  # sparse
        cases.append((rng.integers(0, 300, n) * 65537 + 5).astype(np.uint32))       # sparse, ties
    for r in cases:
        out = np.full(max(len(r), 1), -1, np.int32)
        assert L.dto_rank_order(ptr(r), len(r), ptr(out)) == 0
        assert np.array_equal(out[:len(r)], np.argsort(r, kind="stable").astype(np.int32))
    assert L.dto_rank_order(None, -1, None) != 0


def test_no_oracle_in_product():
    # the product package never imports, includes or links the oracle
    pkg = os.path.join(ROOT, "dual_threshold_optimization_gb300")
    pat = re.compile(r"^\s*(import\s+oracle|from\s+oracle|#\s*include\s*[<\"].*oracle)|liboracle",
                     re.M)
    for dp, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".cpp", ".h")):
                txt = open(os.path.join(dp, f), errors="ignore").read()
                assert not pat.search(txt), f


def test_rust_binding_matches_the_header():
    # the Rust crate (not compiled in this image: no cargo) declares every
    # entry point of include/dto.h, and its structs list the fields in the
    # order of the ctypes binding
    import re
    from dual_threshold_optimization_gb300._lib import DtoResult, DtoSummary
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    hdr = open(os.path.join(root, "include", "dto.h")).read()
    rs = open(os.path.join(root, "dual_threshold_optimization_gb300", "rust", "src", "ffi.rs")).read()
    declared = set(re.findall(r"DTO_API[^(]*?\b(dto_\w+)\(", hdr))
    bound = set(re.findall(r"pub fn (dto_\w+)\(", rs))
    assert declared == bound, (declared ^ bound)

    def fields(struct):
        body = re.search(r"pub struct %s \{(.*?)\n\}" % struct, rs, re.S).group(1)
        return re.findall(r"pub (\w+):", body)
    assert fields("dto_result") == [f for f, _ in DtoResult._fields_]
    assert fields("dto_summary") == [f for f, _ in DtoSummary._fields_]
