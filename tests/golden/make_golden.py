"""Generate tests/golden/reference_golden.json from the reference project.

Run once in a checkout that has the reference project next to it:

    python tests/golden/make_golden.py /path/to/reference

It copies the reference's own test inputs (test_data/ranklist1.csv,
test_data/ranklist2.csv, test_data/background.txt) and records the expected
outputs stated by the reference's tests, doctests and README, each with the
file:line it comes from.  The expected values are typed in from those lines;
nothing here runs reference code (the reference is a Rust crate that cannot be
built without cargo).  The GPU tests read only the JSON this script writes.
"""
import json
import os
import sys


def read_csv(path):
    rows = []
    with open(path) as fh:
        for line in fh:
            line = line.rstrip("\n")
            if not line:
                continue
            g, r = line.split(",")
            rows.append([g.strip(), int(r.strip())])
    return rows


def main(ref):
    td = os.path.join(ref, "test_data")
    with open(os.path.join(td, "background.txt")) as fh:
        background = [ln.strip() for ln in fh if ln.strip()]
    golden = {
        "source": "reference project test_data/, README.md, inline tests and doctests",
        "test_data": {
            "ranklist1": read_csv(os.path.join(td, "ranklist1.csv")),
            "ranklist2": read_csv(os.path.join(td, "ranklist2.csv")),
            "background": background,
            # README.md:173-184 (CLI on test_data, no background, -p 5)
            "expected": {"rank1": 24, "rank2": 13, "set1_len": 24, "set2_len": 13,
                         "population_size": 30, "unpermuted_intersection_size": 12,
                         "unpermuted_pvalue": 0.15632183908046102,
                         "cite": "README.md:173-184"},
        },
        # src/dto/optimize_main.rs:125-170: 10 genes, unpermuted optimum
        "optimize_10": {
            "genes1": ["gene%d" % i for i in range(1, 11)],
            "ranks1": list(range(1, 11)),
            "genes2": ["gene7", "gene3", "gene9", "gene1", "gene5", "gene10", "gene4", "gene8",
                       "gene6", "gene2"],
            "ranks2": list(range(1, 11)),
            "population": 10,
            "expected": {"rank1": 3, "rank2": 4, "pvalue": 0.33333333333333337},
            "cite": "src/dto/optimize_main.rs:128-170",
        },
        # src/stat_operations/hypergeometric_pvalue.rs
        "hypergeometric": [
            {"args": [1000, 50, 60, 10], "p": 0.00044068070222441115, "exact_eq_in_ref": True,
             "cite": "src/stat_operations/hypergeometric_pvalue.rs:27-28"},
            {"args": [6060, 5808, 154, 153], "p": 0.010413637619010246, "exact_eq_in_ref": True,
             "cite": "src/stat_operations/hypergeometric_pvalue.rs:30-31"},
            {"args": [3, 1, 1, 1], "p": 0.3333333333333333, "abs_tol": 1e-10,
             "cite": "src/stat_operations/hypergeometric_pvalue.rs:59-60"},
            {"args": [3, 1, 2, 1], "p": 0.6666666666666666, "abs_tol": 1e-10,
             "cite": "src/stat_operations/hypergeometric_pvalue.rs:63-64"},
            {"args": [3, 1, 3, 1], "p": 1.0, "abs_tol": 1e-10,
             "cite": "src/stat_operations/hypergeometric_pvalue.rs:67-68"},
            {"args": [3, 2, 1, 1], "p": 0.6666666666666666, "abs_tol": 1e-10,
             "cite": "src/stat_operations/hypergeometric_pvalue.rs:74-75"},
            {"args": [3, 2, 2, 2], "p": 0.3333333333333333, "abs_tol": 1e-10,
             "cite": "src/stat_operations/hypergeometric_pvalue.rs:78-79"},
            {"args": [10, 1, 1, 0], "p": 1.0, "abs_tol": 1e-10,
             "cite": "src/stat_operations/hypergeometric_pvalue.rs:85-86"},
        ],
        # src/stat_operations/fdr.rs:20-27
        "fdr": [{"args": [200, 150, 50, 1000, 0.8], "value": 0.240625, "abs_tol": 1e-4,
                 "cite": "src/stat_operations/fdr.rs:20-27"}],
        # src/stat_operations/empirical_pvalue.rs:44-107
        "empirical": {
            "unpermuted": {"rank1": 1, "rank2": 2, "pvalue": 0.05, "set1_len": 50, "set2_len": 40,
                           "population_size": 100, "intersection_size": 10},
            "permuted_pvalues": [0.10, 0.03, 0.07],
            "expected": {"rank1": 1, "rank2": 2, "set1_len": 50, "set2_len": 40,
                         "population_size": 100, "unpermuted_intersection_size": 10,
                         "unpermuted_pvalue": 0.05, "empirical_pvalue": 0.3333333333333333,
                         "fdr": 1.03125},
            "cite": "src/stat_operations/empirical_pvalue.rs:44-107",
        },
        # src/dto/process_threshold_pairs.rs:35-68: 3 thresholds x 3 thresholds
        "grid_3x3": {"ranks1": [1, 2, 3], "ranks2": [1, 2, 3], "records": 9,
                     "cite": "src/dto/process_threshold_pairs.rs:35-68"},
        # src/dto/compute_population_size.rs:111-258
        "population": [
            {"l1": ["gene1", "gene2", "gene3"], "l2": ["gene1", "gene2", "gene4"], "bg": None,
             "error": "If no background is provided, the feature lists must have identical genes.",
             "cite": "src/dto/compute_population_size.rs:111-134"},
            {"l1": ["gene1", "gene2", "gene3"], "l2": ["gene1", "gene2", "gene3"],
             "bg": ["gene1", "gene2"],
             "error": "The following genes in the first ranked feature list are not in the background:",
             "cite": "src/dto/compute_population_size.rs:136-168"},
            {"l1": ["gene1", "gene2", "gene3"], "l2": ["gene1", "gene2", "gene4"],
             "bg": ["gene1", "gene2", "gene3"],
             "error": "The following genes in the second ranked feature list are not in the background:",
             "cite": "src/dto/compute_population_size.rs:170-202"},
            {"l1": ["gene1", "gene2", "gene3"], "l2": ["gene1", "gene2", "gene3"],
             "bg": ["gene1", "gene2", "gene3", "gene4"], "value": 4,
             "cite": "src/dto/compute_population_size.rs:204-235"},
            {"l1": ["gene1", "gene2", "gene3"], "l2": ["gene1", "gene2", "gene3"], "bg": None,
             "value": 3, "cite": "src/dto/compute_population_size.rs:237-258"},
        ],
        # README.md:289-301: the threshold series (the README's claim that the last
        # threshold is forced to the maximum rank does not hold in
        # src/collections/ranked.rs:369-374, which the series below follows)
        "thresholds_prefix": [1, 2, 3, 98, 99, 100, 102, 104],
        "thresholds_cite": "README.md:289-301, src/collections/ranked.rs:359-375",
    }
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_golden.json")
    with open(out, "w") as fh:
        json.dump(golden, fh, indent=1)
    print(out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py REFERENCE_CHECKOUT")
    main(sys.argv[1])
