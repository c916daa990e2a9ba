"""The emulated random streams the reference's genealogy depends on
(never-seeded glibc drand48, glibc rand() after srand(rank+1)), checked
against this machine's libc, and Philox4x32-10 against the published
known-answer vectors of Salmon et al. (Random123)."""
import ctypes as C

import numpy as np
import pytest

libc = C.CDLL("libc.so.6")
libc.drand48.restype = C.c_double


def test_drand48_matches_libc_from_zero_state(orc):
    d = orc.D48()
    orc.lib().orc_drand48_init_default(C.byref(d))
    libc.seed48((C.c_ushort * 3)(0, 0, 0))
    a = [orc.lib().orc_drand48_next(C.byref(d)) for _ in range(2000)]
    b = [libc.drand48() for _ in range(2000)]
    assert a == b
    assert a[0] == 11 / 2**48


def test_drand48_jump_ahead(orc):
    d = orc.D48()
    orc.lib().orc_drand48_init_default(C.byref(d))
    seq = [orc.lib().orc_drand48_next(C.byref(d)) for _ in range(600)]
    for n in (0, 1, 37, 599):
        e = orc.D48()
        orc.lib().orc_drand48_init_default(C.byref(e))
        orc.lib().orc_drand48_skip(C.byref(e), C.c_uint64(n))
        assert orc.lib().orc_drand48_next(C.byref(e)) == seq[n]


@pytest.mark.parametrize("seed", [1, 2, 3, 4, 17, 2**31 - 1])
def test_glibc_rand_matches_libc(orc, seed):
    g = orc.GlibcRand()
    orc.lib().orc_glibc_srand(C.byref(g), seed)
    libc.srand(seed)
    assert [orc.lib().orc_glibc_rand_next(C.byref(g)) for _ in range(5000)] == [libc.rand() for _ in range(5000)]


KAT = [((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
       ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
       ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
        (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1))]


@pytest.mark.parametrize("ctr,key,expect", KAT)
def test_philox_known_answers(orc, ctr, key, expect):
    out = (C.c_uint32 * 4)()
    orc.lib().orc_philox4x32_10((C.c_uint32 * 4)(*ctr), (C.c_uint32 * 2)(*key), out)
    assert tuple(out) == expect


def test_philox_uniform_range(orc):
    u = np.array([orc.philox_uniform(7, i, 1, 2, 3) for i in range(4000)])
    assert (u >= 0).all() and (u < 1).all()
    assert abs(u.mean() - 0.5) < 0.02
