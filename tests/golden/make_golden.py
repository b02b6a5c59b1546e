"""Generates the RNG known-answer fixtures in tests/golden/rng_kat.json from
pure-Python statements of the published generators the reference cites:
xoroshiro64* (prng.di.unimi.it/xoroshiro64star.c, random.glsl:9-26), the
Thomas Wang 32-bit hash (random.glsl:28-38) and the PCG hash (O'Neill 2014;
Jarzynski & Olano 2020).  Independent of the C++ oracle on purpose.

Run: python tests/golden/make_golden.py
"""
import json
import os

M32 = 0xFFFFFFFF


def rotl(x, k):
    return ((x << k) | (x >> (32 - k))) & M32


def wang(s):
    s = (s ^ 61) ^ (s >> 16)
    s = (s * 9) & M32
    s = s ^ (s >> 4)
    s = (s * 0x27D4EB2D) & M32
    s = s ^ (s >> 15)
    return s


def xoroshiro64star(s0, s1, n):
    out = []
    for _ in range(n):
        out.append((s0 * 0x9E3779BB) & M32)
        s1 ^= s0
        s0 = rotl(s0, 26) ^ s1 ^ ((s1 << 9) & M32)
        s1 = rotl(s1, 13)
    return out, (s0, s1)


def pcg_hash(v):
    state = (v * 747796405 + 2891336453) & M32
    word = (((state >> ((state >> 28) + 4)) ^ state) * 277803737) & M32
    return (word >> 22) ^ word


def pcg_stream(state, n):
    out = []
    for _ in range(n):
        state = (state * 747796405 + 2891336453) & M32
        word = (((state >> ((state >> 28) + 4)) ^ state) * 277803737) & M32
        out.append((word >> 22) ^ word)
    return out


def main():
    seeds = [(0, 0), (1, 0), (0, 1), (17, 3), (255, 255), (1919, 1079), (65535, 4095), (12345, 67890)]
    draws = 16
    cases = []
    for px, fr in seeds:
        # rng_init (random.glsl:40-50): s = (wang((x<<16)|y), wang(frame)), one draw discarded;
        # here the seed pair is (pixel id, frame) with pixel id = (x<<16)|y already packed.
        _, st = xoroshiro64star(wang(px), wang(fr), 1)
        x_out, _ = xoroshiro64star(st[0], st[1], draws)
        p_out = pcg_stream(pcg_hash((pcg_hash(px) + fr) & M32), draws)
        cases.append({"seed": [px, fr], "xoroshiro64star": x_out, "pcg": p_out})
    hashes = {"wang": [[v, wang(v)] for v in [0, 1, 61, 0xDEADBEEF, 0xFFFFFFFF, 123456789]],
              "pcg": [[v, pcg_hash(v)] for v in [0, 1, 61, 0xDEADBEEF, 0xFFFFFFFF, 123456789]]}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "rng_kat.json")
    with open(path, "w") as f:
        json.dump({"draws": draws, "streams": cases, "hashes": hashes,
                   "source": "tests/golden/make_golden.py (pure-Python statements of the published generators)"},
                  f, indent=1)
    print(path)


if __name__ == "__main__":
    main()
