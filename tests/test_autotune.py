"""The autotuner's table logic and the committed tuning table (no GPU): entries merge
and order as the library's first-match lookups expect, the header it writes parses back
to the same table, and the compiled-in header agrees with tuning.json when both exist."""
import json
import re
from pathlib import Path

from networksolvers_gb300 import autotune as at

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "networksolvers_gb300"


def parse_header(text):
    tri = re.search(r"kTri\[\] = \{(.*?)\};", text, re.S).group(1)
    split = re.search(r"kSplit\[\] = \{(.*?)\};", text, re.S).group(1)
    tri_e = [tuple(map(int, m)) for m in re.findall(r"\{(-?\d+), (-?\d+)\}", tri)]
    split_e = [tuple(map(int, m)) for m in re.findall(r"\{(-?\d+), (-?\d+), (-?\d+)\}", split)]
    return tri_e, split_e


def test_entries_and_header_round_trip():
    rows = [{"order": 32, "best": 2}, {"order": 64, "best": 4}, {"order": 96, "best": 4},
            {"order": 128, "best": 8}, {"order": 192, "best": -1}, {"order": 256, "best": 16}]
    tri = at.tri_entries(rows)
    assert tri == [(32, 2), (96, 4), (128, 8)]  # merged, and cut at the first grid-kernel order
    srows = [{"tiles": 4, "k": 128, "ms": {"1": 2.0, "2": 1.0}},
             {"tiles": 1, "k": 64, "ms": {"1": 1.0, "2": 1.5}},
             {"tiles": 1, "k": 4096, "ms": {"16": 0.5, "32": 0.4}},
             # a second output size with the same tile count: the summed time decides
             {"tiles": 1, "k": 4096, "ms": {"16": 0.5, "32": 0.7}}]
    split = at.split_entries(srows)
    assert split == [(1, 64, 1), (1, 4096, 16), (4, 128, 2)]
    assert parse_header(at.header(tri, split, "test")) == (tri, split)


def test_cluster_fit_rule_matches_library():
    # (ceil(n/C) n + 4 n) 8 bytes <= 200 KB, as tridiag_cluster checks
    assert at.cluster_fits(360, 16) and not at.cluster_fits(640, 16) and not at.cluster_fits(256, 2)


def test_committed_table_parses_and_matches_json():
    tri, split = parse_header((PKG / "csrc" / "tuning_table.h").read_text())
    assert tri and split
    assert all(a < b for (a, _), (b, _) in zip(tri, tri[1:]))
    assert all(p in (2, 4, 8, 16) for _, p in tri)
    js = PKG / "tuning.json"
    if js.exists():
        d = json.loads(js.read_text())
        assert [tuple(x) for x in d["table"]["tridiag"]] == tri
        assert [tuple(x) for x in d["table"]["splitk"]] == split


def test_rewrite_tables_from_saved_measurements(tmp_path):
    # the committed measurements rewrite to the committed header (no GPU needed)
    js = PKG / "tuning.json"
    if not js.exists():
        return
    assert at.main(["--from-json", str(js), "--out", str(tmp_path)]) == 0
    assert parse_header((tmp_path / "tuning_table.h").read_text()) == parse_header(
        (PKG / "csrc" / "tuning_table.h").read_text())
