"""Loaders for the committed golden fixtures (tests/golden/*.json.gz)."""
import gzip
import json
from functools import lru_cache
from pathlib import Path

GOLDEN = Path(__file__).resolve().parent / "golden"


@lru_cache(maxsize=None)
def utest():
    with gzip.open(GOLDEN / "wfa2_utest.json.gz", "rt") as f:
        return json.load(f)


@lru_cache(maxsize=None)
def ref_cases():
    with gzip.open(GOLDEN / "wfa2_ref_cases.json.gz", "rt") as f:
        return json.load(f)["cases"]


def printed_line(score: int, cigar: str) -> str:
    """align_benchmark's `score\\tCIGAR` line (benchmark_utils.c:103-117)."""
    return f"{score}\t{cigar if cigar else '-'}"
