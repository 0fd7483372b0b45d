"""Readers mirroring the reference's ``src/read``.

read_ranked_feature_list_from_csv  src/read/read_ranked_feature_list_from_csv.rs:50-70
read_feature_list_from_file        src/read/read_feature_list_from_file.rs:45-53
"""
from .feature_lists import Feature, FeatureList, RankedFeatureList


class ReadError(ValueError):
    """The reference panics on unreadable input; this is raised instead."""


def read_ranked_feature_list_from_csv(filepath):
    """Two comma-separated fields per line (feature, rank), no header.  The rank
    is parsed as a non-negative integer and stored as u32."""
    try:
        fh = open(filepath)
    except OSError as e:
        raise ReadError("Could not open file") from e
    genes, ranks = [], []
    with fh:
        for i, line in enumerate(fh):
            line = line.rstrip("\n").rstrip("\r")
            fields = line.split(",")
            if len(fields) != 2:
                raise ReadError("Invalid format in file %s at line %d" % (filepath, i + 1))
            rank_s = fields[1].strip()
            if not rank_s.isdigit():
                raise ReadError("Invalid rank value")
            genes.append(Feature(fields[0].strip()))
            ranks.append(int(rank_s) & 0xFFFFFFFF)
    return RankedFeatureList.from_(FeatureList(genes), ranks)


def read_feature_list_from_file(filepath):
    """One feature id per line (trimmed)."""
    try:
        fh = open(filepath)
    except OSError as e:
        raise ReadError("Could not open file") from e
    with fh:
        return FeatureList([Feature(line.strip()) for line in fh.read().splitlines()])
