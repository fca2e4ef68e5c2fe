"""Small pure-Python M31 / QM31 / circle helpers for known-answer tests (slow; tiny sizes only)."""
P = (1 << 31) - 1


def add(a, b):
    return (a + b) % P


def sub(a, b):
    return (a - b) % P


def mul(a, b):
    return a * b % P


def inv(a):
    return pow(a, P - 2, P)


def cm_mul(x, y):
    return ((x[0] * y[0] - x[1] * y[1]) % P, (x[0] * y[1] + x[1] * y[0]) % P)


def q_add(x, y):
    return tuple((a + b) % P for a, b in zip(x, y))


def q_sub(x, y):
    return tuple((a - b) % P for a, b in zip(x, y))


def q_mul(x, y):
    a, b, c, d = (x[0], x[1]), (x[2], x[3]), (y[0], y[1]), (y[2], y[3])
    ac, bd = cm_mul(a, c), cm_mul(b, d)
    rbd = ((2 * bd[0] - bd[1]) % P, (bd[0] + 2 * bd[1]) % P)
    ad, bc = cm_mul(a, d), cm_mul(b, c)
    return ((ac[0] + rbd[0]) % P, (ac[1] + rbd[1]) % P, (ad[0] + bc[0]) % P, (ad[1] + bc[1]) % P)


def q_m(x, m):
    return tuple(v * m % P for v in x)


def q(v):
    return (v % P, 0, 0, 0)


def padd(p, q_):
    return ((p[0] * q_[0] - p[1] * q_[1]) % P, (p[0] * q_[1] + p[1] * q_[0]) % P)


GEN = (2, 1268011823)


def index_to_point(i):
    r, g = (1, 0), GEN
    i &= (1 << 31) - 1
    while i:
        if i & 1:
            r = padd(r, g)
        g = padd(g, g)
        i >>= 1
    return r


def brev(i, log):
    return int(format(i, f"0{log}b")[::-1], 2) if log else 0


def canonic_half(log):
    """(initial_index, step_size, log_size) of CanonicCoset(log).half_coset()."""
    return (1 << (31 - (log + 1)), 1 << (31 - (log - 1)), log - 1)


def domain_index(half, i):
    init, step, log = half
    n = 1 << log
    if i < n:
        return (init + step * i) & ((1 << 31) - 1)
    return (-(init + step * (i - n))) & ((1 << 31) - 1)


def domain_points_bitrev(half):
    L = half[2] + 1
    return [index_to_point(domain_index(half, brev(r, L))) for r in range(1 << L)]


def rand_m31(rng, n):
    import numpy as np

    out = rng.integers(0, P, size=n, dtype=np.int64)
    return out.astype(np.uint32)
