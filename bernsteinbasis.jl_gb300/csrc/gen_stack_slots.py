"""Generate bbdg_stack_slots.cuh: where each lift-stack entry lives in shared memory.

The stage kernel's chain thread of face f stores stack entry q (layer d, face node (i, j),
q = ijk(N, i, j, d)) of its element; the gather thread of coefficient n reads, for each face f,
the entry p_f(n) (the face permutations of src/BernsteinLift.jl:207-218; p_3(n) = n). The gather's
64-bit loads are served 16 lanes at a time, and lanes 16m..16m+15 always hold coefficients
n = 16m'..16m'+15. Two of those lanes hit the same bank group when their entries are equal mod 16,
so the entries are placed at slots s(q) with slot residues that differ, as far as possible,
within every such block of every face: a min-conflicts search over residues mod 16 (each residue
used at most ceil(Np/16) + 1 times), then s(q) = 16 * (rank of q within its residue) + residue.
All chains store the same slot in their own stacks, so the stores stay conflict-free.

Run: python gen_stack_slots.py > bbdg_stack_slots.cuh   (deterministic; degrees 9 and 10)
"""
import random

# Degrees of the specialised stage kernels with enough gather conflicts to matter (at N = 5 the
# switch also kept the compiler from unrolling the chain into registers).
DEGREES = (9, 10)


def tri(n, j):
    return j * (2 * n + 3 - j) // 2


def tet(n, k):
    a, b = n + 1, n + 1 - k
    return (a * (a + 1) * (a + 2) - b * (b + 1) * (b + 2)) // 6


def ijk(n, i, j, k):
    return i + tri(n, j) + tet(n, k) - j * k


def blocks_of(N):
    NP = (N + 1) * (N + 2) * (N + 3) // 6
    nodes = [(i, j, k) for k in range(N + 1) for j in range(N + 1 - k) for i in range(N + 1 - j - k)]

    def pf(f, n):
        i, j, k = nodes[n]
        l = N - i - j - k
        return (ijk(N, i, k, j), ijk(N, j, k, l), ijk(N, j, k, i), n)[f]

    return NP, [[pf(f, n) for n in range(b, min(b + 16, NP))] for f in range(4) for b in range(0, NP, 16)]


def conflicts(sets, col):
    tot = 0
    for s in sets:
        cnt = {}
        for q in s:
            cnt[col[q]] = cnt.get(col[q], 0) + 1
        tot += max(cnt.values()) - 1
    return tot


def search(N, seed, iters=60000):
    NP, sets = blocks_of(N)
    member = [[] for _ in range(NP)]
    for si, s in enumerate(sets):
        for q in s:
            member[q].append(si)
    rng = random.Random(seed)
    col = [q % 16 for q in range(NP)]
    cap = (NP + 15) // 16 + 1
    counts = [col.count(c) for c in range(16)]

    def clash(q, c):
        return sum(1 for si in member[q] for x in sets[si] if x != q and col[x] == c)

    best, best_col = conflicts(sets, col), list(col)
    for it in range(iters):
        q = rng.randrange(NP)
        if clash(q, col[q]) == 0 and rng.random() < 0.9:
            continue
        opts = sorted((clash(q, c) + (0 if counts[c] < cap or c == col[q] else 99), rng.random(), c)
                      for c in range(16))
        c = opts[0][2]
        if c != col[q]:
            counts[col[q]] -= 1
            counts[c] += 1
            col[q] = c
        if it % 2000 == 0:
            cur = conflicts(sets, col)
            if cur < best:
                best, best_col = cur, list(col)
    cur = conflicts(sets, col)
    if cur < best:
        best, best_col = cur, list(col)
    return best, best_col, conflicts(sets, [q % 16 for q in range(NP)])


def slots(N):
    best = None
    for seed in range(4):
        r = search(N, seed)
        if best is None or r[0] < best[0]:
            best = r
    extra, col, ident = best
    rank = [0] * 16
    out = []
    for q, c in enumerate(col):
        out.append(16 * rank[c] + c)
        rank[c] += 1
    return out, extra, ident


def main():
    print("// Generated by gen_stack_slots.py; do not edit. Lift-stack entry q of degree N lives at")
    print("// slot stack_slot<N>(q) of its stack (see the generator for how the slots were chosen).")
    print("#pragma once")
    print("")
    print("template <int N>")
    print("__host__ __device__ __forceinline__ constexpr int stack_slot(int q) { return q; }")
    print("template <int N>")
    print("struct StackSlots {")
    print("  static constexpr int span = (N + 1) * (N + 2) * (N + 3) / 6;  // slots used: 0..span-1")
    print("};")
    for N in DEGREES:
        s, extra, ident = slots(N)
        span = max(s) + 1
        print("")
        print(f"// N = {N}: modelled extra wavefronts of the gather per element and chain pair: {extra} "
              f"(identity placement: {ident})")
        print("template <>")
        print(f"__host__ __device__ __forceinline__ constexpr int stack_slot<{N}>(int q) {{")
        print("  switch (q) {")
        for q, v in enumerate(s):
            if v != q:
                print(f"    case {q}: return {v};")
        print("    default: return q;")
        print("  }")
        print("}")
        print("template <>")
        print(f"struct StackSlots<{N}> {{")
        print(f"  static constexpr int span = {span};")
        print("};")


if __name__ == "__main__":
    main()
