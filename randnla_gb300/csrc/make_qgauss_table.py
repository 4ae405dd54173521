"""Writes rnla_qgauss_table.h: a Walker alias table for the discretized
standard Gaussian used by the tensor-core sketch.

Target distribution: t = round(8 g) clamped to [-63, 63], g ~ N(0, 1), i.e.
P(t) = Phi((t + 1/2) / 8) - Phi((t - 1/2) / 8) for |t| < 63 and the two
clamped tails for t = +-63.  The probabilities are rounded to integer
weights W_t summing to 2^25 (largest remainders), then Vose's alias
construction in exact integer arithmetic gives 128 buckets of capacity
2^18.  A 32-bit word u samples it as

    b = u >> 25, x = (u >> 7) & (2^18 - 1), e = table[b]
    o = x < (e & (2^18 - 1)) ? (e >> 18) & 127 : e >> 25,   t = o - 63

so P(t) = W_t / 2^25 exactly.  Run once; the header is committed.
"""
import math
import os

N = 128            # buckets (7 bits of the word)
CAP_BITS = 18      # threshold bits
TOTAL = N << CAP_BITS   # 2^25
OFF = 63


def phi(x):
    return 0.5 * math.erfc(-x / math.sqrt(2.0))


def target():
    p = []
    for t in range(-OFF, OFF + 1):
        if t == -OFF:
            v = phi((t + 0.5) / 8.0)
        elif t == OFF:
            v = 0.5 * math.erfc((t - 0.5) / 8.0 / math.sqrt(2.0))
        else:
            v = phi((t + 0.5) / 8.0) - phi((t - 0.5) / 8.0)
        p.append(v)
    return p


def weights(p):
    raw = [v * TOTAL for v in p]
    w = [int(math.floor(r)) for r in raw]
    rem = TOTAL - sum(w)
    order = sorted(range(len(p)), key=lambda i: (-(raw[i] - w[i]), i))
    for i in order[:rem]:
        w[i] += 1
    assert sum(w) == TOTAL
    return w + [0]          # outcome 127: weight 0


def alias_table(w):
    cap = 1 << CAP_BITS
    s = list(w)
    thr = [0] * N
    ali = [0] * N
    small = [o for o in range(N) if s[o] < cap]
    large = [o for o in range(N) if s[o] >= cap]
    while small and large:
        lo = small.pop()
        g = large.pop()
        thr[lo] = s[lo]
        ali[lo] = g
        s[g] -= cap - s[lo]
        (small if s[g] < cap else large).append(g)
    for o in small + large:          # full buckets: always the bucket's own outcome
        thr[o] = 0
        ali[o] = o
    return thr, ali


def check(w, thr, ali):
    cap = 1 << CAP_BITS
    got = [0] * N
    for b in range(N):
        got[b] += thr[b]
        got[ali[b]] += cap - thr[b]
    assert got == w, "alias table does not reproduce the weights"


def main():
    p = target()
    w = weights(p)
    thr, ali = alias_table(w)
    check(w, thr, ali)
    words = [thr[b] | (b << CAP_BITS) | (ali[b] << 25) for b in range(N)]
    lines = []
    for i in range(0, N, 6):
        lines.append("    " + ", ".join("0x%08xu" % v for v in words[i:i + 6]) + ",")
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "rnla_qgauss_table.h"), "w") as f:
        f.write("""// Generated by make_qgauss_table.py -- do not edit.
// Walker alias table of t = round(8 g) clamped to [-63, 63], g ~ N(0, 1):
// P(t) = W_t / 2^25 with integer weights W_t.  Entry b packs the threshold
// (bits 0-17), the bucket's own outcome o = t + 63 (bits 18-24) and its
// alias outcome (bits 25-31).  The table is the definition of the distribution.
#pragma once
#define RNLA_QGAUSS_INIT {\\
""")
        f.write("\\\n".join(lines) + "\\\n}\n")
        f.write("/* sum of W_t t^2 / 2^25 (variance of t) = %.17g */\n" %
                (sum(w[o] * (o - OFF) ** 2 for o in range(127)) / TOTAL))
    print("wrote rnla_qgauss_table.h; nonzero outcomes:", sum(1 for v in w if v))


if __name__ == "__main__":
    main()
