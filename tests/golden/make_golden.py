"""Writes tests/golden/reference_kats.json from the reference's own tests.

Two sources, both in spearfish v0.3.2:

* the known-answer tests of ``crates/map/src/align.rs`` and
  ``crates/map/src/lib.rs`` (transcribed below, each with its file:line), and
* the shrunk failure inputs proptest saved in
  ``crates/map/proptest-regressions/align.txt`` (parsed from the file).

Run in a checkout that has the reference next to it:
``python tests/golden/make_golden.py /path/to/spearfish``.  The JSON it writes is
committed; tests read only the JSON.
"""
from __future__ import annotations

import json
import os
import re
import sys

A, Cc, G, T = 0, 1, 2, 3
MAX_U32 = 0xFFFFFFFF
USIZE_MAX = None  # JSON null: no band / no cut


def codes(s: str) -> list[int]:
    return ["ACGT".index(ch) for ch in s]


def kats() -> list[dict]:
    ont = [2, 4, 4, 2]
    hifi = [1, 4, 6, 2]
    out: list[dict] = []

    def add(fn, args, want, cite, **extra):
        d = {"fn": fn, "args": args, "want": want, "cite": cite}
        d.update(extra)
        out.append(d)

    # align.rs:2908-2926 `examples`
    q, t7 = [0, 1, 2, 3], [3, 3, 0, 1, 2, 3, 3]
    add("distance", {"p": q, "t": t7, "mode": "Infix", "k": MAX_U32}, 0, "align.rs:2910")
    add("distance", {"p": q, "t": [0, 1, 3], "mode": "Infix", "k": MAX_U32}, 1, "align.rs:2911")
    add("distance", {"p": q, "t": [], "mode": "Infix", "k": MAX_U32}, 4, "align.rs:2912")
    add("distance", {"p": q, "t": t7, "mode": "Prefix", "k": 10}, 2, "align.rs:2913-2916")
    add("distance", {"p": q, "t": t7, "mode": "Global", "k": 10}, 3, "align.rs:2917-2920")
    add("distance", {"p": q, "t": t7, "mode": "Global", "k": 2}, None, "align.rs:2921-2924")
    add("distance", {"p": [], "t": [0, 1], "mode": "Global", "k": 5}, 2, "align.rs:2925")

    # align.rs:3169-3180 `affine_examples`
    p8 = [0, 1, 2, 3, 0, 1, 2, 3]
    t10 = [0, 1, 2, 3, 0, 1, 2, 3, 2, 2]
    add("affine", {"p": p8, "t": p8, "mode": "Global", "sc": ont, "band": USIZE_MAX}, 16,
        "align.rs:3173")
    add("affine", {"p": p8, "t": t10, "mode": "Global", "sc": ont, "band": USIZE_MAX}, 8,
        "align.rs:3176")
    add("affine", {"p": p8, "t": t10, "mode": "Prefix", "sc": ont, "band": USIZE_MAX}, 16,
        "align.rs:3177")
    add("affine", {"p": [], "t": [0, 1], "mode": "Global", "sc": ont, "band": USIZE_MAX}, -8,
        "align.rs:3178")
    add("affine", {"p": [0, 1], "t": [], "mode": "Global", "sc": ont, "band": USIZE_MAX}, -8,
        "align.rs:3179")

    # align.rs:3118-3129 `affine_extend_examples`: equal to the naive definition.
    add("affine_extend_vs_naive",
        {"p": [0, 1, 2, 3, 0, 1, 3, 3, 3, 3, 3], "t": [0, 1, 2, 3, 0, 1, 2, 3], "sc": ont,
         "band": USIZE_MAX, "end_bonus": 0, "xdrop": 2 ** 31 - 1}, "naive_extend",
        "align.rs:3123-3127")
    add("affine_extend", {"p": [], "t": [0, 1, 2, 3, 0, 1, 2, 3], "sc": ont, "band": USIZE_MAX,
                          "end_bonus": 0, "xdrop": 2 ** 31 - 1}, 0, "align.rs:3128")

    # align.rs:3131-3143 `affine_extend_end_examples` (window = text length, band 16, xdrop 50)
    t = [0, 1, 2, 3, 0, 1, 2, 3, 0, 1]
    add("affine_extend_end", {"p": [0, 1, 2, 3, 0, 1, 3, 3, 3, 3, 3], "t": t, "sc": ont,
                              "band": 16, "end_bonus": 0, "xdrop": 50}, [12, 6, 6],
        "align.rs:3139")
    add("affine_extend_end", {"p": [0, 1, 2, 0, 1, 2, 3], "t": t, "sc": ont, "band": 16,
                              "end_bonus": 5, "xdrop": 50}, [14 - 6 + 5, 7, 8], "align.rs:3141")
    add("affine_extend_end", {"p": [3, 3, 3], "t": [0, 0, 0], "sc": ont, "band": 16,
                              "end_bonus": 0, "xdrop": 50}, [0, 0, 0], "align.rs:3143")

    # align.rs:3147-3163 `affine_extend_window_cuts` (relations; inputs below)
    tw = [((i * 5 + i // 4) % 4) for i in range(140)]
    pw = tw[:70] + [[3, 3, 0, 0][i % 4] for i in range(40)]
    add("affine_extend_window_cuts", {"p": pw, "t": tw, "sc": ont, "band": 16, "end_bonus": 5,
                                      "xdrop": 30}, "relation", "align.rs:3147-3163")
    # align.rs:3166-3181 `affine_extend_end_reads_a_prefix`
    tr = [((i * 7 + i // 3) % 4) for i in range(120)]
    pr = tr[:60] + [[3, 3, 0, 0][i % 4] for i in range(40)]
    add("affine_extend_end_reads_a_prefix", {"p": pr, "t": tr, "sc": ont, "band": 16,
                                             "end_bonus": 5, "xdrop": 30}, "relation",
        "align.rs:3166-3181")

    # align.rs:3017-3043 `local_band_examples`
    tl = [3, 3, 0, 1, 2, 3, 0, 1, 2, 2, 2]
    pl = [0, 1, 2, 3, 0, 1]
    junk = [2, 2, 2, 0, 1, 2, 3, 0, 1, 3, 3, 3]
    for (p, tt, dlo, dhi, b, want, cite) in [
        (pl, tl, 2, 2, (5, 5), 22, "align.rs:3022"),
        (pl, tl, -6, 11, (5, 5), 22, "align.rs:3023"),
        (pl, tl, 0, 0, (0, 0), 0, "align.rs:3025"),
        (pl, tl, 6, 6, (0, 0), 6, "align.rs:3026"),
        (junk, tl, -12, 11, (5, 5), 12, "align.rs:3029"),
        ([4, 4, 4], [0, 0, 0], -3, 3, (0, 0), 0, "align.rs:3031"),
        ([], tl, -3, 3, (5, 5), 0, "align.rs:3032"),
        (pl, tl, 3, 2, (5, 5), 0, "align.rs:3033"),
        (pl, tl, 2, 2, (5, 0), 17, "align.rs:3035"),
        (pl, tl, 2, 2, (0, 3), 15, "align.rs:3036"),
        ([0, 1, 2, 2], [0, 1, 2], 0, 0, (0, 5), 6, "align.rs:3038"),
        ([0, 1, 2, 2], [0, 1, 2], 0, 0, (5, 0), 11, "align.rs:3039-3042"),
    ]:
        add("local_band_ends", {"p": p, "t": tt, "sc": ont, "dlo": dlo, "dhi": dhi,
                                "bonus": list(b)}, want, cite)

    # crates/map/src/lib.rs:3236-3300 `paper_example_segments_and_per_transcript_scores`:
    # per hit (left extension, interior gap, right extension) with TieBreak defaults
    # (band 16, end_bonus 5, xdrop 50; lib.rs:233-240).  Texts and anchor blocks per hit from
    # lib.rs:3238-3250; left sides are aligned reversed (lib.rs:3266-3274).
    qs = "ACGTATGCACGATCTCAGTA"
    texts = [qs, "GACGTATGCACGATCTCAGT", "ACGTATGCACATGATCTCAGT", "ACGTACGTGCACGATCTCAGT"]
    blocks = [((7, 10), (10, 18)), ((8, 11), (11, 19)), ((7, 10), (12, 20)), ((9, 12), (12, 20))]
    want = [(19, 0, 9), (19, 0, 2), (19, -8, 2), (11, 0, 2)]
    for i in range(4):
        tx = codes(texts[i])
        (b0s, b0e), (b1s, b1e) = blocks[i]
        add("segment_scores", {
            "left_p": codes(qs[:7])[::-1], "left_t": tx[:b0s][::-1],
            "gap_t": tx[b0e:b1s], "right_p": codes(qs[18:]), "right_t": tx[b1e:],
            "sc": ont, "band": 16, "end_bonus": 5, "xdrop": 50}, list(want[i]),
            "map/src/lib.rs:3257-3297")
    add("segment_totals", {}, [28, 21, 13, 13], "map/src/lib.rs:3293")
    # The same example through `Mapper::segmented` (lib.rs:3294-3297): the read, the four
    # transcripts, each hit's chain of (query start, transcript start, length) anchors
    # (lib.rs:3245-3250), TieBreak defaults with flank_min 0 and end_bonus_cut off
    # (lib.rs:3259-3263); costs are the negated totals.
    add("segmented", {"read": codes(qs), "texts": [codes(t) for t in texts],
                      "hits": [[0, [[7, 7, 3], [10, 10, 8]]], [1, [[7, 8, 3], [10, 11, 8]]],
                               [2, [[7, 7, 3], [10, 12, 8]]], [3, [[7, 9, 3], [10, 12, 8]]]],
                      "tb": {"flank_min": 0, "end_bonus_cut": False}},
        [-28, -21, -13, -13], "map/src/lib.rs:3294-3297")
    # `shared_blocks` (lib.rs:562-630): blocks as [[qs, qe], [[ts, te], ...]], None as null.
    for chains, want, cite in (
            ([[[2, 2, 3]], [[2, 2, 4]]], None, "map/src/lib.rs:3164"),
            ([[[2, 4, 3], [2, 8, 4]], [[2, 9, 4]]], [[[2, 6], [[8, 12], [9, 13]]]],
             "map/src/lib.rs:3165-3172"),
            ([[[2, 4, 5], [4, 6, 2], [6, 8, 5], [11, 15, 2]],
              [[2, 5, 5], [4, 7, 2], [6, 9, 5], [11, 16, 2]]],
             [[[2, 11], [[4, 13], [5, 14]]], [[11, 13], [[15, 17], [16, 18]]]],
             "map/src/lib.rs:3173-3190"),
            ([[[2, 2, 5], [4, 5, 5]]], [[[2, 7], [[2, 7]]]], "map/src/lib.rs:3196-3199"),
            ([[[2, 2, 3], [6, 4, 3]]], [[[2, 5], [[2, 5]]]], "map/src/lib.rs:3200-3203"),
            ([[[0, 0, 1], [2, 2, 4], [2, 2, 3], [2, 2, 3], [8, 8, 2], [12, 12, 2]],
              [[1, 2, 1], [2, 3, 3], [2, 3, 4], [7, 8, 1], [12, 15, 2]],
              [[2, 4, 4], [2, 4, 3], [10, 12, 1], [12, 16, 2]]],
             [[[2, 6], [[2, 6], [3, 7], [4, 8]]], [[12, 14], [[12, 14], [15, 17], [16, 18]]]],
             "map/src/lib.rs:3207-3229"),
            ([[[0, 0, 1], [2, 2, 4], [2, 2, 3], [2, 2, 3], [8, 8, 2], [12, 12, 2]], []], None,
             "map/src/lib.rs:3230-3232")):
        add("shared_blocks", {"chains": chains}, want, cite)
    # `tail_start` (lib.rs:2935-2969) with run 15 (lib.rs:3307-3313).
    for seq, want, cite in (("CGTCAAAAAAAAAAAAAAAGT", [4, 19], "map/src/lib.rs:3309"),
                            ("CGAAAAAAACAAAAAAAGT", [2, 17], "map/src/lib.rs:3311"),
                            ("CGTCAAAAAAAAAAGTCAAAA", None, "map/src/lib.rs:3312")):
        add("tail_start", {"rest": codes(seq), "run": 15}, want, cite)
    _ = hifi
    return out


def regressions(path: str) -> list[dict]:
    """Parses proptest's saved shrink cases: `cc <hash> # shrinks to a = .., b = ..`."""
    cases = []
    with open(path) as f:
        for line in f:
            m = re.match(r"cc ([0-9a-f]+) # shrinks to (.*)$", line.strip())
            if not m:
                continue
            args = eval("dict(" + m.group(2) + ")", {"__builtins__": {}, "dict": dict})
            keys = set(args)
            if keys == {"p", "t", "k"}:
                test = "random_vs_naive"
            elif keys == {"t", "edits", "a", "len", "slack"}:
                test = "related_vs_naive"
            elif keys == {"p", "t", "bonus"}:
                test = "local_band_matches_definition"
            elif "variants" in keys and "base" in keys:
                test = "sorted_batch_matches_single"
            elif "seed" in keys:
                test = "narrow_cells_match_wide"
            else:
                test = "unknown"
            # JSON-friendly: tuples to lists.
            cases.append({"test": test, "hash": m.group(1), "args": json.loads(json.dumps(args)),
                          "cite": "crates/map/proptest-regressions/align.txt"})
    return cases


def main() -> None:
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <reference checkout (the spearfish source tree)>")
    ref = sys.argv[1]
    reg = regressions(os.path.join(ref, "crates/map/proptest-regressions/align.txt"))
    doc = {"source": "COMBINE-lab/spearfish v0.3.2",
           "note": "KATs transcribed from the reference tests (cite = file:line); regressions "
                   "parsed from its proptest-regressions file.  Codes: A0 C1 G2 T3.",
           "kats": kats(), "regressions": reg}
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_kats.json")
    with open(out, "w") as f:
        json.dump(doc, f, indent=1)
    print(out, len(doc["kats"]), "kats", len(reg), "regressions")


if __name__ == "__main__":
    main()
