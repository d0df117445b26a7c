"""Philox4x32-10 of the oracle against the generator's published
known-answer vectors (Salmon et al., SC'11; Random123 kat_vectors)."""
from tests import oracle_lib

KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


def test_philox_known_answers():
    for ctr, key, want in KAT:
        assert tuple(oracle_lib.philox_raw(ctr, key)) == want


def test_step_words_layout():
    seed = 0x0123456789ABCDEF
    block = 0x00000002FFFFFFFF
    got = oracle_lib.step_words(seed, block, 7)
    want = oracle_lib.philox_raw((block & 0xFFFFFFFF, block >> 32, 7, 0),
                                 (seed & 0xFFFFFFFF, seed >> 32))
    assert got == want


def test_host_philox_matches_oracle():
    from jmmonedmc_gb300.philox_host import philox4x32_10
    for ctr, key, want in KAT:
        assert philox4x32_10(*ctr, *key) == want
    assert list(philox4x32_10(5, 0, 9, 0, 1, 0)) == oracle_lib.philox_raw((5, 0, 9, 0), (1, 0))
