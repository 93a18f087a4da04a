"""NumPy restatement of Philox4x32-10 (Salmon et al., SC'11) and of the
engine's uniform / Box-Muller mapping, for checking the device RNG."""
import numpy as np

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = np.uint64(0x9E3779B9), np.uint64(0xBB67AE85)
MASK = np.uint64(0xFFFFFFFF)


def philox4x32_10(ctr, key):
    """ctr: (N, 4) uint32, key: (2,) uint32 -> (N, 4) uint32."""
    c = [np.asarray(ctr[:, i], dtype=np.uint64) for i in range(4)]
    k0, k1 = np.uint64(key[0]), np.uint64(key[1])
    for r in range(10):
        if r > 0:
            k0 = (k0 + W0) & MASK
            k1 = (k1 + W1) & MASK
        p0 = M0 * c[0]
        p1 = M1 * c[2]
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK
        c = [hi1 ^ c[1] ^ k0, lo1, hi0 ^ c[3] ^ k1, lo0]
    return np.stack([x.astype(np.uint32) for x in c], axis=1)


def raw(count, seed, counter):
    pairs = (count + 1) // 2
    e = np.arange(pairs, dtype=np.uint64)
    ctr = np.stack([e & MASK, e >> np.uint64(32), np.full(pairs, counter & 0xFFFFFFFF, np.uint64),
                    np.full(pairs, (counter >> 32) & 0xFFFFFFFF, np.uint64)], axis=1).astype(np.uint32)
    key = np.array([seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF], dtype=np.uint32)
    return philox4x32_10(ctr, key)


def _u53(a, b):
    return ((a >> 5).astype(np.float64) * 67108864.0 + (b >> 6).astype(np.float64)) / 9007199254740992.0


def uniform(count, seed, counter):
    r = raw(count, seed, counter)
    out = np.stack([_u53(r[:, 0], r[:, 1]), _u53(r[:, 2], r[:, 3])], axis=1).reshape(-1)
    return out[:count]


def normal(count, seed, counter):
    """Box-Muller of the fp32-rounded inputs fp32(1 - u) and fp32(v), here in
    float64; the device evaluates the same formula in fp32 (~1e-7 apart)."""
    r = raw(count, seed, counter)
    u, v = _u53(r[:, 0], r[:, 1]), _u53(r[:, 2], r[:, 3])
    x = (1.0 - u).astype(np.float32).astype(np.float64)
    t = 2.0 * v.astype(np.float32).astype(np.float64)
    rad = np.sqrt(-2.0 * np.log(x))
    out = np.stack([rad * np.cos(np.pi * t), rad * np.sin(np.pi * t)], axis=1).reshape(-1)
    return out[:count]
