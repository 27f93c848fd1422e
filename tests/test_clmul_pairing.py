"""The device GF(2^128) product's 32 x 32 carry-less step (field.cuh, clmul32_classes)
sums pairs of same-class hole products as integers (in the multiply's addend) and XORs
the rest. This checks that arithmetic on the CPU against a bitwise carry-less multiply:
random operands, dense operands and the all-ones worst case (8 + 7 partial products in a
column)."""
import random

MASK32 = [0x11111111, 0x22222222, 0x44444444, 0x88888888]
MASK64 = [0x1111111111111111, 0x2222222222222222, 0x4444444444444444, 0x8888888888888888]
U64 = (1 << 64) - 1


def clmul_ref(x, y):
    r = 0
    for i in range(32):
        if (y >> i) & 1:
            r ^= x << i
    return r


def clmul_paired(x, y):
    X = [x & m for m in MASK32]
    Y = [y & m for m in MASK32]
    mw = lambda a, b: (a * b) & U64
    madw = lambda a, b, c: (a * b + c) & U64
    z0 = madw(X[0], Y[0], mw(X[1], Y[3])) ^ mw(X[2], Y[2]) ^ mw(X[3], Y[1])
    z1 = madw(X[0], Y[1], mw(X[2], Y[3])) ^ madw(X[1], Y[0], mw(X[3], Y[2]))
    z2 = madw(X[0], Y[2], mw(X[3], Y[3])) ^ mw(X[1], Y[1]) ^ mw(X[2], Y[0])
    z3 = mw(X[0], Y[3]) ^ mw(X[1], Y[2]) ^ mw(X[2], Y[1]) ^ mw(X[3], Y[0])
    return (z0 & MASK64[0]) | (z1 & MASK64[1]) | (z2 & MASK64[2]) | (z3 & MASK64[3])


def test_paired_hole_products_match_carryless_multiply():
    rng = random.Random(20260)
    cases = [(0xFFFFFFFF, 0xFFFFFFFF), (0xFFFFFFFF, 0), (0x88888888, 0x88888888), (0x11111111, 0xFFFFFFFF),
             (0xFFFF0000, 0x0000FFFF), (1, 1), (0x80000000, 0x80000000)]
    for _ in range(20000):
        a, b = rng.getrandbits(32), rng.getrandbits(32)
        if rng.random() < 0.3:
            a |= rng.getrandbits(32) | rng.getrandbits(32)
        if rng.random() < 0.3:
            b |= rng.getrandbits(32) | rng.getrandbits(32)
        cases.append((a, b))
    bad = [(a, b) for a, b in cases if clmul_paired(a, b) != clmul_ref(a, b)]
    assert not bad, bad[:5]
