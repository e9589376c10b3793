"""Pure-Python Philox4x32-10 (Salmon et al., SC'11), used by the tests to
reproduce the device random stream bit for bit."""
M0, M1 = 0xD2511F53, 0xCD9E8D57
W0, W1 = 0x9E3779B9, 0xBB67AE85
MASK = 0xFFFFFFFF


def philox4x32_10(ctr, key):
    c0, c1, c2, c3 = ctr
    k0, k1 = key
    for _ in range(10):
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = (p0 >> 32) & MASK, p0 & MASK
        hi1, lo1 = (p1 >> 32) & MASK, p1 & MASK
        c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
        k0 = (k0 + W0) & MASK
        k1 = (k1 + W1) & MASK
    return c0, c1, c2, c3


def below(v, n):
    return (v * n) >> 32


def random_states_ref(n_batches, N, n_down, seed, sid):
    """Mirror of the vmck_random_states kernel."""
    import numpy as np
    k0, k1 = seed & MASK, (seed >> 32) & MASK
    out = np.empty((n_batches, N), dtype=np.int8)
    for b in range(n_batches):
        if n_down < 0:
            for base in range(0, N, 128):
                r = philox4x32_10((b & MASK, (b >> 32) & MASK, base >> 7, sid & MASK), (k0, k1))
                for i in range(base, min(N, base + 128)):
                    bit = (r[(i - base) >> 5] >> ((i - base) & 31)) & 1
                    out[b, i] = -1 if bit else 1
            continue
        row = [(-1 if i < n_down else 1) for i in range(N)]
        r = None
        q = 0
        for i in range(N - 1, 0, -1):
            if q % 4 == 0:
                r = philox4x32_10((b & MASK, (b >> 32) & MASK, q >> 2, (sid ^ 0x80000000) & MASK),
                                  (k0, k1))
            j = below(r[q % 4], i + 1)
            row[i], row[j] = row[j], row[i]
            q += 1
        out[b] = row
    return out
