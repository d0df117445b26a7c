"""Host-side Philox4x32-10 (the same generator as csrc/philox.cuh), used to
draw per-chain workload parameters (pressures, temperatures) from a seed."""

_M0, _M1 = 0xD2511F53, 0xCD9E8D57
_W0, _W1 = 0x9E3779B9, 0xBB67AE85
_MASK = 0xFFFFFFFF


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    for _ in range(10):
        p0 = _M0 * c0
        p1 = _M1 * c2
        c0, c1, c2, c3 = ((p1 >> 32) ^ c1 ^ k0) & _MASK, p1 & _MASK, \
                         ((p0 >> 32) ^ c3 ^ k1) & _MASK, p0 & _MASK
        k0 = (k0 + _W0) & _MASK
        k1 = (k1 + _W1) & _MASK
    return c0, c1, c2, c3


def uniforms(seed, count, stream=0):
    """`count` uniforms in [0, 1): word 0 of blocks (i, 0, stream, 0xffffffff)."""
    k0, k1 = seed & _MASK, (seed >> 32) & _MASK
    return [philox4x32_10(i & _MASK, i >> 32, stream, 0xFFFFFFFF, k0, k1)[0] / 4294967296.0
            for i in range(count)]
