"""Derives the characteristic polynomial of the MT19937 state transition and prints it as the C
table `kMtCharTerms` used by probes.cu.

MT19937's transition is linear over GF(2) and its characteristic polynomial χ has degree 19937 and
is primitive, so every nonzero output bit sequence has minimal polynomial χ.  Berlekamp–Massey
on 2·19937 consecutive bits of one bit position of the untempered words recovers it; the script
prints the exponents of its nonzero terms.  Run: python gen_mt_charpoly.py
"""
from __future__ import annotations

N = 624
DEG = 19937


def seed_state(s: int) -> list[int]:
    st = [s & 0xFFFFFFFF]
    for i in range(1, N):
        st.append((1812433253 * (st[-1] ^ (st[-1] >> 30)) + i) & 0xFFFFFFFF)
    return st


def extend(x: list[int], count: int) -> list[int]:
    """Appends `count` words: x[j] = x[j−227] ⊕ twist(upper bit of x[j−624] | lower 31 of x[j−623])."""
    for _ in range(count):
        j = len(x)
        y = (x[j - 624] & 0x80000000) | (x[j - 623] & 0x7FFFFFFF)
        x.append(x[j - 227] ^ (y >> 1) ^ (0x9908B0DF if y & 1 else 0))
    return x


def berlekamp_massey(bits: list[int]) -> tuple[int, int]:
    """Connection polynomial C (bit i = c_i, c_0 = 1) and linear complexity L over GF(2)."""
    C, B, L, m, R = 1, 1, 0, 1, 0
    for n, s in enumerate(bits):
        R = (R << 1) | s           # bit i of R = s_{n−i}
        if (C & R).bit_count() & 1 == 0:
            m += 1
        elif 2 * L <= n:
            C, B, L, m = C ^ (B << m), C, n + 1 - L, 1
        else:
            C ^= B << m
            m += 1
    return C, L


def char_terms(seed: int = 5489, bit: int = 0) -> list[int]:
    x = extend(seed_state(seed), 2 * DEG)
    C, L = berlekamp_massey([(w >> bit) & 1 for w in x[N:N + 2 * DEG]])
    if L != DEG:
        raise RuntimeError(f"linear complexity {L} != {DEG}")
    # χ(z) = z^L C(1/z): coefficient of z^(L−i) is c_i
    return sorted(L - i for i in range(L + 1) if (C >> i) & 1)


if __name__ == "__main__":
    t = char_terms()
    body = ",".join(str(v) for v in t)
    print(f"// {len(t)} terms, degree {t[-1]}")
    print(f"constexpr int kMtCharTerms[{len(t)}] = {{{body}}};")
