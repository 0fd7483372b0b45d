"""Seeded synthetic ranked-list pairs.

No public dataset stands behind the reference's profiling runs (its
"long" input files are not shipped), so every workload here is synthetic:

* list-1 ranks: a seeded random permutation of 1..N;
* list-2 ranks: a Gaussian copula with correlation rho to list 1,
  z1 = Phi^-1(rank1 / (N + 1)), z2 = rho z1 + sqrt(1 - rho^2) eps, rank2 =
  ordinal rank of z2;
* ties by the "min" method: the list's rank order is cut into consecutive
  blocks and every member of a block gets the block's smallest rank.

The named workloads follow the benchmark configurations: N = 6,000 with 10%
of list-2 features in tie blocks of size 2-5 (rho 0.3); N = 20,000 without
ties (rho 0.2); 25,000-feature rankings restricted to an 18,000-feature
background with geometric tie blocks (mean size 5, rho 0.1); and batches of
pairs with N and rho drawn uniformly.
"""
import numpy as np
from scipy.special import ndtri


class ListPair:
    """Two ranked lists over dense feature ids, plus names for CSV output."""

    def __init__(self, ranks1, feat1, ranks2, feat2, n_features, population, names=None):
        self.ranks1 = np.asarray(ranks1, np.uint32)
        self.feat1 = np.asarray(feat1, np.int32)
        self.ranks2 = np.asarray(ranks2, np.uint32)
        self.feat2 = np.asarray(feat2, np.int32)
        self.n_features = int(n_features)
        self.population = int(population)
        self.names = names

    def feature_names(self):
        if self.names is None:
            self.names = ["g%d" % f for f in range(self.n_features)]
        return self.names

    def sorted_lists(self):
        """(ranks, features) of each list after the stable sort by rank."""
        o1 = np.argsort(self.ranks1, kind="stable")
        o2 = np.argsort(self.ranks2, kind="stable")
        return (self.ranks1[o1], self.feat1[o1]), (self.ranks2[o2], self.feat2[o2])


def min_method_ties(ranks, rng, frac_tied=0.0, block_sizes=(2, 5), geometric_p=None):
    """Collapse consecutive runs of the rank order into tie blocks (min method).

    frac_tied: approximate fraction of features that end up in blocks of
    uniform size in block_sizes; geometric_p: instead, partition the whole
    order into blocks of Geometric(p) size.
    """
    ranks = np.asarray(ranks, np.int64)
    order = np.argsort(ranks, kind="stable")
    out = ranks.copy()
    n = len(ranks)
    pos = 0
    lo, hi = block_sizes
    mean_block = (lo + hi) / 2.0
    start_prob = frac_tied / (mean_block * (1.0 - frac_tied) + frac_tied) if frac_tied > 0 else 0.0
    while pos < n:
        if geometric_p is not None:
            size = int(rng.geometric(geometric_p))
        elif start_prob > 0 and rng.random() < start_prob:
            size = int(rng.integers(lo, hi + 1))
        else:
            size = 1
        size = min(size, n - pos)
        block = order[pos:pos + size]
        out[block] = ranks[order[pos]]
        pos += size
    return out


def copula_pair(N, rho, seed, frac_tied2=0.0, geometric_p=None):
    """A no-background pair over N shared features."""
    rng1 = np.random.default_rng(seed)
    rng2 = np.random.default_rng(seed + 1)
    rank1 = rng1.permutation(N) + 1
    z1 = ndtri(rank1 / (N + 1.0))
    z2 = rho * z1 + np.sqrt(1.0 - rho * rho) * rng2.standard_normal(N)
    rank2 = np.empty(N, np.int64)
    rank2[np.argsort(z2, kind="stable")] = np.arange(1, N + 1)
    if geometric_p is not None:
        rank1 = min_method_ties(rank1, rng2, geometric_p=geometric_p)
        rank2 = min_method_ties(rank2, rng2, geometric_p=geometric_p)
    elif frac_tied2 > 0:
        rank2 = min_method_ties(rank2, rng2, frac_tied=frac_tied2)
    feats = np.arange(N, dtype=np.int32)
    return ListPair(rank1, feats, rank2, feats.copy(), N, N)


def background_pair(universe, background, rho, seed, geometric_p=0.2):
    """Two universe-sized copula rankings restricted to a seeded background
    subset; ranks keep their universe values (gaps), ties in geometric blocks.
    Population = background size."""
    rng = np.random.default_rng(seed + 7)
    full = copula_pair(universe, rho, seed, geometric_p=geometric_p)
    keep = np.sort(rng.choice(universe, size=background, replace=False))
    r1 = full.ranks1[keep]
    r2 = full.ranks2[keep]
    feats = np.arange(background, dtype=np.int32)
    return ListPair(r1, feats, r2, feats.copy(), background, background)


def config1():
    """N = 6,000, rho 0.3, ~10% of list-2 features in tie blocks of size 2-5."""
    return copula_pair(6000, 0.3, seed=1, frac_tied2=0.10)


def config2():
    """N = 20,000, rho 0.2, no ties."""
    return copula_pair(20000, 0.2, seed=2)


def config4():
    """25,000-feature rankings restricted to an 18,000-feature background,
    geometric tie blocks of mean size 5, rho 0.1."""
    return background_pair(25000, 18000, 0.1, seed=4, geometric_p=0.2)


def batch_pairs(count=512, n_lo=2000, n_hi=30000, rho_lo=0.0, rho_hi=0.4, seed=3):
    """Uneven batch: N ~ U[n_lo, n_hi], rho ~ U[rho_lo, rho_hi] per pair."""
    rng = np.random.default_rng(seed)
    ns = rng.integers(n_lo, n_hi + 1, size=count)
    rhos = rng.uniform(rho_lo, rho_hi, size=count)
    return [copula_pair(int(n), float(r), seed=int(seed * 100003 + q)) for q, (n, r) in enumerate(zip(ns, rhos))]


def small_pair(N, rho, seed, frac_tied2=0.0, subset1=None, subset2=None):
    """A small pair for parity tests; optional subsets make the two lists
    cover different features (background mode)."""
    p = copula_pair(N, rho, seed, frac_tied2=frac_tied2)
    if subset1 is None and subset2 is None:
        return p
    rng = np.random.default_rng(seed + 11)
    k1 = np.sort(rng.choice(N, size=subset1 or N, replace=False))
    k2 = np.sort(rng.choice(N, size=subset2 or N, replace=False))
    return ListPair(p.ranks1[k1], p.feat1[k1], p.ranks2[k2], p.feat2[k2], N, N)
