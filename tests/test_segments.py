"""The reduction-segment rule is stated twice: in the device code (dev.h,
red_segments: four-tile segments up to kSegSplit tiles, one-tile segments
above, at most kRedSegs) and in the oracle's mirror of the GPU's summation
order (ldu_oracle.c, mr_reduce).  Bit-identical results depend on both
agreeing; this reads the constants from both sources and checks the rule on
the sizes the tests and the workloads use."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _const(path, pattern):
    txt = open(os.path.join(ROOT, path)).read()
    m = re.search(pattern, txt)
    assert m, (path, pattern)
    return int(m.group(1))


def test_segment_rule_matches_oracle_mirror():
    dev = "multiregionfoam_gb300/csrc/dev.h"
    orc = "oracle/ldu_oracle.c"
    red = _const(dev, r"constexpr int kRedSegs = (\d+);")
    tiles = _const(dev, r"constexpr int kSegTiles = (\d+);")
    split = _const(dev, r"constexpr int kSegSplit = (\d+);")
    assert red == _const(orc, r"#define MR_GRID (\d+)")
    assert tiles == _const(orc, r"#define MR_SEG_TILES (\d+)")
    assert split == _const(orc, r"#define MR_SEG_SPLIT (\d+)")

    def segments(t):
        g = t if t > split else (t + tiles - 1) // tiles
        return max(1, min(red, g))

    # 1560 cells (2 tiles), C1 (94), the 64^3 GAMG case (256), a 435k-cell
    # system (425), C3 (720), C2 (3072)
    assert [segments(t) for t in (2, 94, 256, 257, 425, 720, 3072)] == [1, 24, 64, 257, 425, 608, 608]
