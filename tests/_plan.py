"""Python restatement of the engine's binomial checkpoint planner (test helper).

Griewank & Walther's binomial reversal ("Algorithm 799: revolve", ACM TOMS
26(1), 2000), in the form of cuda_fwi_gb300/csrc/fwi_host.cpp (plan_binomial):
the state of step 0 is the zero state (no slot), `slots` states can be held.
recompute_after_first_sweep() is the number of forward steps the backward
runs once forward() has placed the SAVEs of the first sweep: from the last of
them to the last step, then every ADVANCE after that prefix.
"""
from __future__ import annotations

import math
import sys


def _beta(S, r):
    return 0 if r < 0 else math.comb(S + r, r)


def binomial_cost(l, s):
    if l <= 1:
        return 0
    S = s + 1
    if s == 0:
        return l * (l - 1) // 2
    r = 0
    while _beta(S, r) < l:
        r += 1
    return r * l - _beta(S + 1, r - 1)


def plan(n, slots):
    out, working, free = [], [0], list(range(slots - 1, -1, -1))

    def advance(a, b):
        if b > a:
            out.append(("A", a, b))
        working[0] = b

    def restore(slot, st):
        if working[0] != st:
            out.append(("R", slot, st))
        working[0] = st

    def rev(a, b, slot, s):
        l = b - a
        if l == 1:
            restore(slot, a)
            out.append(("J", a))
            return
        if s == 0:
            for i in range(b - 1, a - 1, -1):
                restore(slot, a)
                advance(a, i)
                out.append(("J", i))
            return
        best, S, r = binomial_cost(l, s), s + 1, 0
        while _beta(S, r) < l:
            r += 1
        j = max(1, l - _beta(S - 1, r))
        while j < l and j + binomial_cost(l - j, s - 1) + binomial_cost(j, s) != best:
            j += 1
        if j >= l:
            j = 1
        m = a + j
        restore(slot, a)
        advance(a, m)
        ms = free.pop()
        out.append(("S", ms, m))
        rev(m, b, ms, s - 1)
        free.append(ms)
        restore(slot, a)
        rev(a, m, slot, s)

    old = sys.getrecursionlimit()
    sys.setrecursionlimit(max(old, 4 * n + 100))
    try:
        if n > 0:
            rev(0, n, -1, slots)
    finally:
        sys.setrecursionlimit(old)
    return out


def recompute_after_first_sweep(n, slots):
    acts = plan(n, slots)
    k, last = 0, 0
    while k < len(acts) and acts[k][0] != "J":
        if acts[k][0] == "S":
            last = acts[k][2]
        k += 1
    return (n - 1 - last) + sum(a[2] - a[1] for a in acts[k:] if a[0] == "A")
