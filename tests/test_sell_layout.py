"""The sliced-ELL layout's arithmetic restated on the CPU, on the Hubbard m=512 superblock of the
reference's own DMRG run (L=64, U=4, the largest superblock of the 4th sweep; built by the oracle,
bitwise the device build): rows sorted by length in windows of 2048, 32-row slices padded to their
longest row, and, for the 16-bit column-delta stream, one zero bridge element per 65,535 columns of
every gap between neighbouring columns of a row beyond the first 65,535.  The two totals are the
ones the device build reported on a GB300 (dg_matrix_format, dg_matrix_sell_deltas);
tests/test_gpu_sell_deltas.py checks the device against this restatement directly."""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import GOLDEN

WINDOW, SLICE, BRIDGE = 2048, 32, 65535
DEVICE_STORED, DEVICE_BRIDGES = 56_362_528, 42_080   # dg_matrix_format / dg_matrix_sell_deltas on a GB300


def row_bridges(indptr, indices):
    """Zero elements each row needs so that every delta between neighbouring columns fits 16 bits."""
    n = len(indptr) - 1
    lens = np.diff(indptr)
    gaps = np.diff(indices.astype(np.int64))
    rowid = np.repeat(np.arange(n), lens)
    inrow = rowid[1:] == rowid[:-1]
    out = np.zeros(n, np.int64)
    np.add.at(out, rowid[1:][inrow], np.maximum(0, (gaps[inrow] - 1) // BRIDGE))
    return out


def sell_stored(lengths):
    """Stored slots of the sliced-ELL layout: length-sorted windows, slices padded to their longest row."""
    n = len(lengths)
    nwin = -(-n // WINDOW)
    padded = np.zeros(nwin * WINDOW, np.int64)
    padded[:n] = lengths
    w = -np.sort(-padded.reshape(nwin, WINDOW), axis=1)          # each window by decreasing length
    return int(SLICE * w.reshape(-1, SLICE).max(axis=1).sum())


@pytest.fixture(scope="module")
def full_m512(oracle):
    from dmrg_c_gb300 import sb_models
    path = GOLDEN / "dmrg_hubbard_vf_sweep4.npz"
    if not path.exists():
        pytest.skip("no Hubbard m=512 superblock fixture")
    sb = sb_models.load_dmrg_superblock(path)
    row, col, val = oracle.sb_build(sb.model)
    n = sb.model.n
    low = sp.csr_matrix((val, col, row), shape=(n, n))
    full = (low + sp.tril(low, -1).T).tocsr()
    full.sort_indices()
    return full


def test_bridges_and_stored_slots_match_the_device_build(full_m512):
    A = full_m512
    assert A.nnz == 56_222_276
    br = row_bridges(A.indptr, A.indices)
    assert int(br.sum()) == DEVICE_BRIDGES
    assert int(br.max()) == 1 and np.mean(br > 0) < 0.2
    assert sell_stored(np.diff(A.indptr) + br) == DEVICE_STORED
    # the plain layout (no bridges) is 0.075 % smaller
    assert sell_stored(np.diff(A.indptr)) < DEVICE_STORED


def test_bridges_on_a_small_case():
    """Hand-checked gaps: 65,535 needs none, 65,536 one, 131,070 one (65,535 + 65,535), 131,072 two."""
    indptr = np.array([0, 2, 4, 6, 8, 9])
    indices = np.array([0, 65535, 0, 65536, 1, 131071, 0, 131072, 7])
    assert row_bridges(indptr, indices).tolist() == [0, 1, 1, 2, 0]
