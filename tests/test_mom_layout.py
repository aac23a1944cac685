"""CPU: the chunked byte layout of the moment storage (LBM_FP16NEQ).

A moment buffer holds, per node, nine 16-bit fields and three byte fields,
in chunks of 64 consecutive nodes of a row (the pitch is a multiple of 256):
inside a chunk the nine 16-bit fields as 128-byte planes, then the three
byte fields as 64-byte planes.  These are the address rules of
parallellbmcranfield_gb300/csrc/lbm_mom.cuh (mom_off, mom_off_lo and the
bulk kernel's per-thread row pointers) restated in numpy, checked for being
a bijection onto the buffer's 21 bytes per node and for the bulk kernel's
shortcut (one pointer per thread and row, every field at a fixed offset)
agreeing with the per-node rule.
"""
import numpy as np
import pytest

CH = 64            # nodes per chunk
CHB = 21 * CH      # bytes per chunk
LO = 18 * CH       # first byte plane inside a chunk


def mom_off(z):
    """Byte offset of node z's slot in 16-bit plane 0 (plane p: + 128 p)."""
    z = np.asarray(z, np.int64)
    return 21 * (z & ~np.int64(CH - 1)) + 2 * (z & (CH - 1))


def mom_off_lo(z):
    """Byte offset of node z's slot in byte plane 0 (plane p: + 64 p)."""
    z = np.asarray(z, np.int64)
    return 21 * (z & ~np.int64(CH - 1)) + LO + (z & (CH - 1))


@pytest.mark.parametrize("pitch,m", [(256, 3), (512, 5), (1280, 2)])
def test_layout_is_a_bijection(pitch, m):
    nodes = np.arange(pitch * m, dtype=np.int64)
    owner = np.full(21 * pitch * m, -1, np.int64)
    for p in range(9):
        for b in range(2):
            idx = mom_off(nodes) + 2 * CH * p + b
            assert (owner[idx] == -1).all()
            owner[idx] = nodes
    for p in range(3):
        idx = mom_off_lo(nodes) + CH * p
        assert (owner[idx] == -1).all()
        owner[idx] = nodes
    assert (owner >= 0).all()  # every byte of the 21 per node is used once
    # each node's bytes lie inside its own 1344-byte chunk
    chunk = np.arange(owner.size) // CHB
    assert (owner // CH == chunk).all()


@pytest.mark.parametrize("pitch", [256, 768, 16384])
def test_row_pointer_shortcut(pitch):
    """The bulk kernel forms mom_off(r * pitch + x0) as r * 21 * pitch +
    mom_off(x0') with x0' = x0 clamped to the row (x0 is even, from -2 up)."""
    rowb = 21 * pitch
    x0 = np.arange(-2, pitch + 62, 2, dtype=np.int64)
    x0c = np.clip(x0, 0, pitch - 2)
    for r in (0, 1, 7, 1000):
        z = r * pitch + x0c
        assert (r * rowb + mom_off(x0c) == mom_off(z)).all()
        assert (r * rowb + mom_off_lo(x0c) == mom_off_lo(z)).all()
        # both nodes of a pair share a chunk: the pair's 32-bit and 16-bit
        # words are whole and aligned
        assert (mom_off(z) % 4 == 0).all() and (mom_off_lo(z) % 2 == 0).all()
        assert ((z // CH) == ((z + 1) // CH)).all()


@pytest.mark.parametrize("pitch", [256, 4096])
def test_prefetch_span_covers_the_warp(pitch):
    """Lanes 0..21 prefetch the 128-byte lines from the first to the last
    chunk that a warp's columns wx - 2 .. wx + 61 touch, clamped to the row."""
    for wx in range(0, pitch, 60):
        pf0 = CHB * (max(wx - 2, 0) // CH)
        pf1 = CHB * (min(wx + 61, pitch - 1) // CH + 1)
        assert 0 <= pf0 < pf1 <= 21 * pitch
        assert pf1 - pf0 <= 2 * CHB  # at most two chunks: 22 lines at a 64-byte offset
        lines = {(min(pf0 + 128 * lane, pf1 - 1)) // 128 for lane in range(22)}
        need = set(range(pf0 // 128, (pf1 - 1) // 128 + 1))
        assert need <= lines
        cols = np.arange(max(wx - 2, 0), min(wx + 62, pitch))
        assert (mom_off(cols) >= pf0).all() and (mom_off_lo(cols) + 2 * CH < pf1).all()
