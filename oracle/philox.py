"""Oracle: Philox4x32-10 counter-based generator (numpy, uint32 exact).

Restates the published algorithm of Salmon, Moraes, Dror and Shaw,
"Parallel random numbers: as easy as 1, 2, 3" (SC'11): ten rounds of two
32x32->64 multiplies with the paper's multipliers and Weyl key increments.
The product's CUDA sampler uses the same counter layout, so given the same
seed the oracle reproduces the exact uniforms the GPU drew. Test
infrastructure only.
"""
import numpy as np

_M0 = np.uint64(0xD2511F53)
_M1 = np.uint64(0xCD9E8D57)
_W0 = np.uint32(0x9E3779B9)
_W1 = np.uint32(0xBB67AE85)
_MASK = np.uint64(0xFFFFFFFF)


def philox4x32(c0, c1, c2, c3, k0, k1):
    """Vectorised over broadcastable uint32 arrays; returns 4 uint32 arrays."""
    c0 = np.asarray(c0, dtype=np.uint32)
    c1 = np.asarray(c1, dtype=np.uint32)
    c2 = np.asarray(c2, dtype=np.uint32)
    c3 = np.asarray(c3, dtype=np.uint32)
    k0 = np.asarray(k0, dtype=np.uint32)
    k1 = np.asarray(k1, dtype=np.uint32)
    c0, c1, c2, c3, k0, k1 = np.broadcast_arrays(c0, c1, c2, c3, k0, k1)
    c0, c1, c2, c3, k0, k1 = (x.copy() for x in (c0, c1, c2, c3, k0, k1))
    with np.errstate(over="ignore"):
        for _ in range(10):
            p0 = _M0 * c0.astype(np.uint64)
            p1 = _M1 * c2.astype(np.uint64)
            hi0 = (p0 >> np.uint64(32)).astype(np.uint32)
            lo0 = (p0 & _MASK).astype(np.uint32)
            hi1 = (p1 >> np.uint64(32)).astype(np.uint32)
            lo1 = (p1 & _MASK).astype(np.uint32)
            c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
            k0 = k0 + _W0
            k1 = k1 + _W1
    return c0, c1, c2, c3


def to_uniform(x):
    """(x >> 8) + 0.5 scaled by 2^-24: exactly representable in float32, in (0, 1)."""
    return ((np.asarray(x, dtype=np.uint32) >> np.uint32(8)).astype(np.float64) + 0.5) * (2.0 ** -24)


def seed_key(seed):
    seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    return np.uint32(seed & 0xFFFFFFFF), np.uint32(seed >> 32)


def ar_site_uniforms(seed, offset, n_samples, n_sites):
    """Uniform for (sample b, site k) of one autoregressive draw: counter
    (b, k, offset_lo, offset_hi), output word 0."""
    k0, k1 = seed_key(seed)
    b = np.arange(n_samples, dtype=np.uint32)[:, None]
    k = np.arange(n_sites, dtype=np.uint32)[None, :]
    off = int(offset) & 0xFFFFFFFFFFFFFFFF
    x0, _, _, _ = philox4x32(b, k, np.uint32(off & 0xFFFFFFFF), np.uint32(off >> 32), k0, k1)
    return to_uniform(x0)


def mh_words(seed, chain, sweep):
    """Four words for (chain, sweep) of a Metropolis-Hastings run: counter
    (chain, sweep_lo, sweep_hi, 0x4D48)."""
    k0, k1 = seed_key(seed)
    sweep = int(sweep)
    return philox4x32(np.asarray(chain, dtype=np.uint32), np.uint32(sweep & 0xFFFFFFFF),
                      np.uint32(sweep >> 32), np.uint32(0x4D48), k0, k1)


def ham_words(seed, chain, sweep):
    """Four words for (chain, sweep) of a Hamiltonian-proposal
    Metropolis-Hastings run: counter (chain, sweep_lo, sweep_hi, 0x484D)."""
    k0, k1 = seed_key(seed)
    sweep = int(sweep)
    return philox4x32(np.asarray(chain, dtype=np.uint32), np.uint32(sweep & 0xFFFFFFFF),
                      np.uint32(sweep >> 32), np.uint32(0x484D), k0, k1)
