"""The CUDA block dvmh_loop_cuda_get_config_C hands a handler: the
reference's choice and limits (rts/dvmh/loop.cpp:2134-2199, default blocks
loop.cpp:1464-1485, device limits dvmh_device.cpp:400-440), through the pure
function the library exports (no GPU needed).  GB300's limits: 1024 threads
per block, 48 KB of shared memory and 65536 registers per block, 255
registers per thread at most."""
import ctypes

import pytest

import __graft_entry__ as ge


class Limits(ctypes.Structure):
    _fields_ = [("maxBlockSize", ctypes.c_int * 3), ("maxThreadsPerBlock", ctypes.c_int),
                ("sharedPerBlock", ctypes.c_long), ("regsPerBlock", ctypes.c_long), ("warpSize", ctypes.c_int),
                ("maxRegsPerThread", ctypes.c_int)]


GB300 = Limits((ctypes.c_int * 3)(1024, 1024, 64), 1024, 49152, 65536, 32, 255)


@pytest.fixture(scope="module")
def pick():
    ge.build()
    _, g = ge.package()
    L = g.runtime()
    L.dvmhgb_pick_block.restype = ctypes.c_int
    L.dvmhgb_pick_block.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int * 3, ctypes.c_long,
                                    ctypes.c_long, ctypes.POINTER(Limits)]

    def f(rank, deps, user, block, shared=0, regs=0):
        b = (ctypes.c_int * 3)(*block)
        rc = L.dvmhgb_pick_block(rank, deps, user, b, shared, regs, ctypes.byref(GB300))
        return rc, tuple(b)
    return f


def test_default_blocks_by_free_dimensions(pick):
    # 256 / 32x8 / 32x4x2 by the block dimensions the loop may use: its rank, one fewer with dependences
    assert pick(1, 0, 0, (0, 0, 0)) == (0, (256, 1, 1))
    assert pick(2, 0, 0, (0, 0, 0)) == (0, (32, 8, 1))
    assert pick(3, 0, 0, (0, 0, 0)) == (0, (32, 4, 2))
    assert pick(4, 0, 0, (0, 0, 0)) == (0, (32, 4, 2))
    assert pick(3, 1, 0, (0, 0, 0)) == (0, (32, 8, 1))
    assert pick(2, 1, 0, (0, 0, 0)) == (0, (256, 1, 1))
    assert pick(1, 1, 0, (0, 0, 0)) == (0, (1, 1, 1))


def test_register_limit_shrinks_a_chosen_block(pick):
    # 255 registers (the default when the handler passes 0) x 256 threads = 65280 fits; x 512 does not:
    # one dimension of min(256, 65536 / 255) rounded down to the warp size
    assert pick(2, 0, 0, (0, 0, 0), regs=255) == (0, (32, 8, 1))
    assert pick(2, 0, 0, (32, 16, 1), regs=255) == (0, (256, 1, 1))
    assert pick(2, 0, 0, (32, 16, 1), regs=0) == (0, (256, 1, 1))
    assert pick(3, 0, 0, (32, 8, 4), regs=128) == (0, (256, 1, 1))
    assert pick(3, 0, 0, (32, 8, 4), regs=64) == (0, (32, 8, 4))       # 1024 x 64 = 65536 fits exactly
    assert pick(1, 0, 0, (1024, 1, 1), regs=200) == (0, (256, 1, 1))  # 65536 / 200 = 327, capped at 256
    assert pick(3, 0, 0, (1024, 1, 1), regs=255) == (0, (256, 1, 1))
    assert pick(2, 1, 0, (512, 1, 1), regs=255) == (0, (256, 1, 1))
    assert pick(1, 1, 0, (1, 1, 1), regs=255) == (0, (1, 1, 1))


def test_shared_limit_shrinks_a_chosen_block(pick):
    # 256 threads x 256 bytes = 64 KB > 48 KB: min(256, 49152 / 256 = 192) threads
    assert pick(2, 0, 0, (32, 8, 1), shared=256, regs=32) == (0, (192, 1, 1))
    # 700 bytes per thread: 49152 / 700 = 70 -> 64 threads
    assert pick(3, 0, 0, (0, 0, 0), shared=700, regs=32) == (0, (64, 1, 1))
    # fits: unchanged
    assert pick(2, 0, 0, (32, 8, 1), shared=64, regs=32) == (0, (32, 8, 1))


def test_user_blocks_are_checked_not_shrunk(pick):
    assert pick(2, 0, 1, (32, 16, 1), regs=255)[0] == 5   # registers insufficient for the user's block
    assert pick(2, 0, 1, (32, 8, 1), shared=256, regs=32)[0] == 4
    assert pick(2, 0, 1, (32, 8, 2))[0] == 1              # more block dimensions than the loop has
    assert pick(3, 1, 1, (8, 8, 4))[0] == 1               # ... minus one with dependences
    assert pick(3, 0, 1, (2048, 1, 1))[0] == 2            # an axis above the device's limit
    assert pick(3, 0, 1, (4, 4, 128))[0] == 2
    assert pick(3, 0, 1, (64, 32, 1), regs=32)[0] == 3    # 2048 threads
    assert pick(3, 0, 1, (32, 4, 2), regs=32) == (0, (32, 4, 2))
