"""Generates fft_layouts.h: the shared-memory layout of every inter-stage exchange of the
register-chained line FFT (fft_line.cuh, line_fft_reg), chosen by a bank model.

A line group is C interleaved lines of length L transformed by C*T threads (thread lt:
line c = lt % C, element offset t = lt / C), E = L/T elements per thread, with the radix plan
of fft_line.cuh (pick_radix). Between two stages every thread stores its E outputs and loads
the next stage's E inputs as 8-byte (float2) shared-memory accesses. The model counts, for
each warp instruction, the wavefronts of its two half-warps (16 lanes x 8 bytes cover the 32
banks once; lanes on the same bank pair with different addresses serialise, equal addresses
broadcast) and picks, per exchange, the layout with the fewest store + load wavefronts
(ties: the first in LAYOUTS). Run: python gen_fft_layouts.py (writes fft_layouts.h beside it).
"""
import os

HERE = os.path.dirname(os.path.abspath(__file__))

# index maps of element a (all below a + a/8 + 1 entries, the size of a line buffer)
LAYOUTS = [
    ("a + a/16", lambda a: a + (a >> 4)),
    ("a + a/16 + 2*(a/32)", lambda a: a + (a >> 4) + 2 * (a >> 5)),
    ("a + a/16 + 4*(a/64)", lambda a: a + (a >> 4) + 4 * (a >> 6)),
    ("a + a/16 + 8*(a/128)", lambda a: a + (a >> 4) + 8 * (a >> 7)),
    ("a ^ ((a/16)%8) ^ (((a/64)%2)*8)", lambda a: a ^ ((a >> 4) & 7) ^ (((a >> 6) & 1) << 3)),
]


def pick_radix(rem, E):
    if rem % 3 == 0 and E % 3 == 0:
        return 3
    for R in (16, 8, 4):
        if rem % R == 0 and E % R == 0:
            return R
    return 2


def plan(L, E):
    st, rem, NS = [], L, 1
    while rem > 1:
        R = pick_radix(rem, E)
        if rem % R or E % R:
            return None
        st.append((R, NS))
        NS *= R
        rem //= R
    return st


def wavefronts(elems):
    tot = 0
    for half in (elems[:16], elems[16:]):
        if half:
            slots = {}
            for e in set(half):
                slots.setdefault(e % 16, set()).add(e)
            tot += max(len(v) for v in slots.values())
    return tot


def exchange_cost(L, T, C, st, k, f):
    """Wavefronts of the stores of stage k and the loads of stage k + 1."""
    (R, NS), (R2, _) = st[k], st[k + 1]
    E = L // T
    nth = C * T
    tot = 0
    for w in range((nth + 31) // 32):
        lanes = range(32 * w, min(32 * w + 32, nth))
        for b in range(E // R):
            for r in range(R):
                tot += wavefronts([f((((lt // C + b * T) // NS) * NS * R + (lt // C + b * T) % NS + r * NS) * C + lt % C)
                                   for lt in lanes])
        for b in range(E // R2):
            for r in range(R2):
                tot += wavefronts([f((lt // C + b * T + r * (L // R2)) * C + lt % C) for lt in lanes])
    return tot


def lengths():
    L = 16
    while L <= 8192:
        yield L
        L *= 2
    L = 48
    while L <= 6144:
        yield L
        L *= 2


def main():
    rows = []
    for L in lengths():
        for E in (4, 6, 8, 12, 16, 24):
            if L % E:
                continue
            T = L // E
            st = plan(L, E)
            if st is None:
                continue
            for C in (1, 2, 4, 8):
                if C * T > 1024:
                    continue
                for k in range(len(st) - 1):
                    costs = [exchange_cost(L, T, C, st, k, f) for _, f in LAYOUTS]
                    best = min(range(len(LAYOUTS)), key=lambda i: (costs[i], i))
                    if best:
                        rows.append((L, E, C, st[k + 1][1], best, costs[0], costs[best]))
    out = ["// Generated by gen_fft_layouts.py (bank model of the line FFT's inter-stage exchanges);",
           "// do not edit. Layout of the exchange that feeds the stage of stride NS of a line FFT",
           "// of length L, E elements per thread, C interleaved lines; 0 (a + a/16) where not listed.",
           "// Modelled wavefronts (a + a/16 -> chosen) in the comment of each entry.",
           "#pragma once", "", "namespace fsim {", "",
           "__host__ __device__ constexpr int fft_xlay(int L, int E, int C, int NS) {"]
    for L, E, C, NS, lay, c0, c1 in rows:
        out.append("  if (L == %d && E == %d && C == %d && NS == %d) return %d;  // %d -> %d" % (L, E, C, NS, lay, c0, c1))
    out += ["  return 0;", "}", "", "}  // namespace fsim", ""]
    with open(os.path.join(HERE, "fft_layouts.h"), "w") as fh:
        fh.write("\n".join(out))
    print("%d exchanges with a layout other than a + a/16" % len(rows))


if __name__ == "__main__":
    main()
