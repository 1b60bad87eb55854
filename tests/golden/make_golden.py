"""Generates tests/golden/rng.json: TEA-64 hashes and LCG rnd() streams of
programs/random.cuh:33-65, computed by a pure-Python statement of the
published algorithms (TEA: Wheeler & Needham 1994; LCG a=1664525,
c=1013904223: Numerical Recipes).  Run: python tests/golden/make_golden.py"""
import json
import os
import struct

M32 = 0xFFFFFFFF


def tea64(v0, v1):
    s0 = 0
    for _ in range(64):
        s0 = (s0 + 0x9E3779B9) & M32
        v0 = (v0 + ((((v1 << 4) + 0xA341316C) & M32) ^ ((v1 + s0) & M32)
                    ^ (((v1 >> 5) + 0xC8013EA4) & M32))) & M32
        v1 = (v1 + ((((v0 << 4) + 0xAD90777D) & M32) ^ ((v0 + s0) & M32)
                    ^ (((v0 >> 5) + 0x7E95761E) & M32))) & M32
    return v0


def f32(x):
    return struct.unpack("f", struct.pack("f", x))[0]


def rnd_stream(seed, n):
    out = []
    for _ in range(n):
        seed = (1664525 * seed + 1013904223) & M32
        out.append(f32((seed & 0xFFFFFF) / 16777216.0))
    return out


def main():
    inputs = [[0, 0], [1, 0], [0, 1], [512 * 17 + 3, 5], [1920 * 1079 + 1919, 127],
              [M32, M32], [123456789, 987654321]]
    seeds = [tea64(a, b) for a, b in inputs[:4]]
    g = {"tea_inputs": inputs, "tea64": [tea64(a, b) for a, b in inputs],
         "lcg_seeds": seeds, "rnd_streams": [rnd_stream(s, 16) for s in seeds]}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "rng.json")
    with open(path, "w") as f:
        json.dump(g, f, indent=1)
    print(path)


if __name__ == "__main__":
    main()
