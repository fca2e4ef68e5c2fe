"""A plain big-integer restatement of the Starknet Poseidon hash (starknet-crypto 0.6.2's published
algorithm: Hades over p = 2^251 + 17 * 2^192 + 1, 8 full + 83 partial rounds, x^3, MDS
[[3, 1, 1], [1, -1, 1], [1, 1, -2]], round constants SHA-256("Hades" || k) mod p) and of the
reference's Poseidon252 hasher and channel, independent of the oracle's C++ (test helper)."""
from hashlib import sha256

P252 = 2 ** 251 + 17 * 2 ** 192 + 1
P31 = (1 << 31) - 1
_ARK = [int(sha256(f"Hades{k}".encode()).hexdigest(), 16) % P252 for k in range(3 * 91)]


def permute(s):
    s = list(s)
    for r in range(91):
        s = [(x + _ARK[3 * r + i]) % P252 for i, x in enumerate(s)]
        if r < 4 or r >= 87:
            s = [pow(x, 3, P252) for x in s]
        else:
            s[2] = pow(s[2], 3, P252)
        a, b, c = s
        s = [(3 * a + b + c) % P252, (a - b + c) % P252, (a + b - 2 * c) % P252]
    return s


def hash2(x, y):
    return permute([x, y, 2])[0]


def hash_many(v):
    s = [0, 0, 0]
    i = 0
    while i + 2 <= len(v):
        s[0] = (s[0] + v[i]) % P252
        s[1] = (s[1] + v[i + 1]) % P252
        s = permute(s)
        i += 2
    rem = len(v) - i
    if rem == 1:
        s[0] = (s[0] + v[i]) % P252
    s[rem] = (s[rem] + 1) % P252
    return permute(s)[0]


def hash_node(children, vals):
    v = list(children) if children else []
    nb = (len(vals) + 7) // 8
    padded = list(vals) + [0] * (8 * nb - len(vals))
    for b in range(nb):
        w = 0
        for x in padded[8 * b:8 * b + 8]:
            w = (w * 2 ** 31 + x) % P252
        v.append(w)
    return hash_many(v)


def trailing_zeros(d):
    be = d.to_bytes(32, "big")
    x = int.from_bytes(be[:16], "little")
    return 128 if x == 0 else (x & -x).bit_length() - 1


class Channel:
    def __init__(self, digest=0):
        self.digest, self.n_sent = digest, 0

    def mix_felts(self, felts):
        res = [self.digest]
        for i in range(0, len(felts), 2):
            cur = 0
            for f in felts[i:i + 2]:
                for y in f:
                    cur = (cur * 2 ** 31 + y) % P252
            res.append(cur)
        self.digest, self.n_sent = hash_many(res), 0

    def draw_base_felts(self):
        cur = hash2(self.digest, self.n_sent)
        self.n_sent += 1
        out = []
        for _ in range(8):
            out.append((cur % 2 ** 31) % P31)
            cur //= 2 ** 31
        return out

    def draw_felts(self, n):
        out = []
        while len(out) < n:
            f = self.draw_base_felts()
            out.append(tuple(f[:4]))
            if len(out) < n:
                out.append(tuple(f[4:]))
        return out
