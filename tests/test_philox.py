"""Philox4x32-10 against the known-answer vectors of the Random123 paper."""
import numpy as np

from oracle.philox import philox4x32, u53

KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF), (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


def test_philox_known_answers():
    for ctr, key, want in KAT:
        got = philox4x32(*ctr, *key)
        assert tuple(int(x) for x in got) == want


def test_philox_vectorised_matches_scalar():
    c0 = np.arange(17, dtype=np.uint64)
    v = philox4x32(c0, 5, 9, 1, 0x1234, 0x5678)
    for i in range(17):
        s = philox4x32(i, 5, 9, 1, 0x1234, 0x5678)
        assert all(int(v[j][i]) == int(s[j]) for j in range(4))


def test_uniform_maps():
    assert u53(0, 0) == 0.0
    assert u53(0xFFFFFFFF, 0xFFFFFFFF) < 1.0
