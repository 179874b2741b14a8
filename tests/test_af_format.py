"""The device VCF formatter's AF (hazard H10): "%.2f" of (float)alt /
(float)(ref + alt) widened to double, which Java rounds HALF_UP on the
shortest decimal digits of the double.  The formatter rounds 100 * f half up
instead (exact in double for a float-valued f); this checks that the two rules
agree: the formatter's arithmetic restated with numpy float32 against the
oracle's Java restatement (shortest round-trip digits, then HALF_UP), for every
pair with a total up to 700 and for random large pairs past float's 24-bit
integer range."""
import math
import os
import random

import numpy as np

from oracle import oracle

SRC = os.path.join(os.path.dirname(__file__), "..", "pilon_gb300", "csrc", "pg_format.cu")


def fmt_af(alt, tot):
    f = np.float32(alt) / np.float32(tot)      # (float)alt / (float)tot, float32 division
    d = float(f) * 100.0                          # exact
    fl = math.floor(d)
    if d - fl >= 0.5:
        fl += 1.0
    v = int(fl)
    return ("-" if v < 0 else "") + f"{abs(v) // 100}.{abs(v) % 100:02d}"


def _java(alt, tot):
    return oracle.java_format2(float(np.float32(alt) / np.float32(tot)))


def test_every_small_pair():
    bad = [(a, t) for t in range(1, 701) for a in range(0, t + 1) if fmt_af(a, t) != _java(a, t)]
    assert not bad, bad[:10]


def test_random_large_pairs():
    rng = random.Random(23)
    for _ in range(20000):
        t = rng.randrange(1, 1 << rng.choice([12, 20, 26, 31]))
        a = rng.randrange(0, t + 1)
        assert fmt_af(a, t) == _java(a, t), (a, t)


def test_kernel_af_lines():
    src = open(SRC).read()
    for line in ["const float f = (float)alt / (float)tot;", "const double d = (double)f * 100.0;  // exact",
                 "if (d - fl >= 0.5) fl += 1.0;"]:
        assert line in src, line
