"""Generate tests/golden/pcg32.json: raw PCG32 outputs of RndSampler(seed, idx) for a
few (seed, idx) pairs, computed with an independent pure-Python PCG32 (the published
XSH-RR generator, seeded as the reference's src/sampler.cpp:3-9). The oracle's C++
restatement is checked against these values."""
import json
import os

M64 = (1 << 64) - 1


def pcg32_stream(seed, idx, n):
    state, inc = 0, (((idx + 1) << 1) | 1) & M64

    def step():
        nonlocal state
        old = state
        state = (old * 6364136223846793005 + inc) & M64
        xs = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        rot = old >> 59
        return ((xs >> rot) | (xs << ((-rot) & 31))) & 0xFFFFFFFF

    step()
    state = (state + 0x853C49E6748FEA9B + seed) & M64
    step()
    return [step() for _ in range(n)]


cases = [{"seed": s, "idx": i, "u32": pcg32_stream(s, i, 8)} for s, i in [(0, 0), (1, 0), (0, 1), (123456789, 65535),
                                                                          (2 ** 63, 7)]]
json.dump({"generator": "PCG32 XSH-RR, RndSampler(seed, idx) seeding", "cases": cases},
          open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "pcg32.json"), "w"), indent=1)
