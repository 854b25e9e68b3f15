"""TEST INFRASTRUCTURE ONLY.  Host (numpy) restatement of the device generators in
pico_gb300/csrc/gen.cu, used by the tests to check that the CUDA generators
produce exactly the documented edge lists."""
import numpy as np

M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def mix64(z):
    z = np.asarray(z, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def _thr(p):
    return min(max(int(np.floor(p * 4294967296.0)), 0), 4294967296)


def rmat(scale, m, seed, a=0.57, b=0.19, c=0.19, threads=1):
    """R-MAT edge list (src, dst); the C restatement for large m (on
    `threads` host threads when threads > 1)."""
    if m > 1 << 20:
        import ctypes
        import oracle
        L = oracle.lib()
        u32p = ctypes.POINTER(ctypes.c_uint32)
        L.orc_gen_rmat.argtypes = [ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                                   ctypes.c_uint64, ctypes.c_uint64, u32p, u32p]
        L.orc_gen_rmat.restype = None
        src = np.empty(m, dtype=np.uint32)
        dst = np.empty(m, dtype=np.uint32)
        if threads > 1:
            L.orc_gen_rmat_mt(scale, m, _thr(a), _thr(a + b), _thr(a + b + c), seed,
                              src.ctypes.data_as(u32p), dst.ctypes.data_as(u32p), int(threads))
        else:
            L.orc_gen_rmat(scale, m, _thr(a), _thr(a + b), _thr(a + b + c), seed,
                           src.ctypes.data_as(u32p), dst.ctypes.data_as(u32p))
        return src, dst
    return rmat_numpy(scale, m, seed, a, b, c)


def rmat_numpy(scale, m, seed, a=0.57, b=0.19, c=0.19):
    i = np.arange(m, dtype=np.uint64)
    with np.errstate(over="ignore"):
        base = mix64(np.uint64(seed) * np.uint64(0xD1B54A32D192ED03) + i)
    ta, tab, tabc = _thr(a), _thr(a + b), _thr(a + b + c)
    u = np.zeros(m, dtype=np.uint64)
    v = np.zeros(m, dtype=np.uint64)
    word = None
    for bit in range(scale):
        if bit % 2 == 0:
            with np.errstate(over="ignore"):
                word = mix64(base ^ (np.uint64((bit >> 1) + 1) * np.uint64(0xA24BAED4963EE407)))
        r = (word >> np.uint64(32 * (bit & 1))) & np.uint64(0xFFFFFFFF)
        q = np.where(r < ta, 0, np.where(r < tab, 1, np.where(r < tabc, 2, 3))).astype(np.uint64)
        u = (u << np.uint64(1)) | (q >> np.uint64(1))
        v = (v << np.uint64(1)) | (q & np.uint64(1))
    return u.astype(np.uint32), v.astype(np.uint32)


class Feistel:
    def __init__(self, N, seed):
        bits = 2
        while bits < 64 and (1 << bits) < N:
            bits += 2
        self.half = bits // 2
        self.mask = np.uint64((1 << self.half) - 1)
        self.N = N
        with np.errstate(over="ignore"):
            self.key = [mix64(np.uint64(seed) * np.uint64(0x9E6C63D0676A9A99) + np.uint64(r + 1))
                        for r in range(4)]

    def once(self, x):
        h = np.uint64(self.half)
        L, R = x >> h, x & self.mask
        for r in range(4):
            F = mix64(self.key[r] ^ R) & self.mask
            L, R = R, L ^ F
        return (L << h) | R

    def perm(self, i):
        x = np.asarray(i, dtype=np.uint64).copy()
        todo = np.ones(x.shape, dtype=bool)
        while todo.any():
            x[todo] = self.once(x[todo])
            todo = x >= np.uint64(self.N)
        return x


def tri_unrank(k, p):
    p = np.asarray(p, dtype=np.uint64)
    kk = float(2 * k - 1)
    disc = kk * kk - 8.0 * p.astype(np.float64)
    ad = (kk - np.sqrt(np.maximum(disc, 0))) / 2.0
    r = np.where(ad > 0, ad, 0).astype(np.uint64)
    r = np.minimum(r, np.uint64(k - 2))
    K = np.uint64(k)
    one, two = np.uint64(1), np.uint64(2)

    def T(x):
        return x * K - x * (x + one) // two
    while True:
        m = (r > 0) & (T(r) > p)
        if not m.any():
            break
        r[m] -= one
    while True:
        m = (r + one <= np.uint64(k - 2)) & (T(r + one) <= p)
        if not m.any():
            break
        r[m] += one
    return r, p - T(r) + r + one


def er(n, m, seed):
    N = n * (n - 1) // 2
    f = Feistel(N, seed)
    p = f.perm(np.arange(m, dtype=np.uint64))
    a, b = tri_unrank(n, p)
    return a.astype(np.uint32), b.astype(np.uint32)


def planted(n, k, prob, seed):
    with np.errstate(over="ignore"):
        f = Feistel(n, np.uint64(seed) ^ np.uint64(0x5851F42D4C957F2D))
    members = f.perm(np.arange(k, dtype=np.uint64)).astype(np.uint32)
    npairs = k * (k - 1) // 2
    p = np.arange(npairs, dtype=np.uint64)
    with np.errstate(over="ignore"):
        h = mix64(np.uint64(seed) * np.uint64(0xC2B2AE3D27D4EB4F) + p) & np.uint64(0xFFFFFFFF)
    sel = p[h < np.uint64(_thr(prob))]
    a, b = tri_unrank(k, sel)
    return members[a.astype(np.int64)], members[b.astype(np.int64)]


def ba(n, d, seed):
    """Barabasi-Albert edge list of pico_gb300/csrc/gen.cu (Batagelj-Brandes
    copy model, each odd slot resolved by following r = hash(slot) % slot)."""
    m = n * d
    k = np.arange(m, dtype=np.uint64)
    slot = 2 * k + np.uint64(1)
    target = np.zeros(m, dtype=np.uint64)
    todo = np.ones(m, dtype=bool)
    for _ in range(4096):
        if not todo.any():
            break
        with np.errstate(over="ignore"):
            r = mix64(np.uint64(seed) * np.uint64(0x9FB21C651E98DF25) + slot[todo]) % slot[todo]
        even = (r & np.uint64(1)) == 0
        idx = np.flatnonzero(todo)
        target[idx[even]] = (r[even] >> np.uint64(1)) // np.uint64(d)
        slot[idx[~even]] = r[~even]
        todo[idx[even]] = False
    return (k // np.uint64(d)).astype(np.uint32), target.astype(np.uint32)


def rmat_bounded(n, m, seed, a=0.57, b=0.19, c=0.19):
    scale = 1
    while (1 << scale) < n:
        scale += 1
    u, v = rmat_numpy(scale, m, seed, a, b, c)
    bad = (u >= n) | (v >= n)
    u[bad] = 0
    v[bad] = 0
    return u, v
