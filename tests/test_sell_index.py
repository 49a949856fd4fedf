"""The element walk of the 16-bit delta kernel (sell_row_acc_d16 in csrc/sell.cuh) restated on the
CPU: a slice of width w is split into chunks of 32 elements dealt to its WS warps in turn; a warp
walks full groups of 8 of its chunks (Q of them), then single elements of the slice's last chunk
when that chunk is partial and belongs to it.  For every width up to 400 and WS in {1, 2, 4, 8}
the warps together take every element once, each in increasing order, restarting the running
column (from the chunk's checkpoint) exactly at the chunk starts it takes; and the streamed form's
stages (8 elements each, sell_tma.cuh) restart at the same elements."""
import pytest

CHUNK, U = 32, 8
GPC = CHUNK // U


def warp_walk(w, ws, sub):
    """(k, restarts_here) for every element warp `sub` of `ws` adds, in its order."""
    nch = (w + CHUNK - 1) // CHUNK
    mine = (nch - sub + ws - 1) // ws if nch > sub else 0
    last = nch - 1
    tail = w - last * CHUNK
    owns_last = mine > 0 and (last - sub) % ws == 0
    Q = (mine - 1) * GPC + tail // U if owns_last else mine * GPC
    out = []
    for q in range(Q):
        k0 = (sub + (q // GPC) * ws) * CHUNK + (q % GPC) * U
        for u in range(U):
            out.append((k0 + u, q % GPC == 0 and u == 0))
    if owns_last and tail % U:
        k = last * CHUNK + (tail // U) * U
        first = True
        while k < w:
            out.append((k, first and tail < U))   # restart only if no full group of the chunk ran
            first = False
            k += 1
    return out


@pytest.mark.parametrize("ws", [1, 2, 4, 8])
def test_every_element_once_in_order(ws):
    for w in range(0, 401):
        seen = []
        for sub in range(ws):
            walk = warp_walk(w, ws, sub)
            ks = [k for k, _ in walk]
            assert ks == sorted(ks), (w, ws, sub)
            for k, restart in walk:
                assert restart == (k % CHUNK == 0), (w, ws, sub, k)
            seen += ks
        assert sorted(seen) == list(range(w)), (w, ws)


def test_one_warp_is_the_plain_order():
    """With one warp a slice the walk is k = 0, 1, ..., w-1: the order of the 32-bit-column kernel
    with 8-element groups, which is why the two are bitwise equal."""
    for w in range(0, 401):
        assert [k for k, _ in warp_walk(w, 1, 0)] == list(range(w))


def test_stages_restart_at_chunk_starts():
    """The streamed form's stage t covers elements 8t .. 8t + 7 (fewer in the last); a stage starts
    a chunk exactly when 8t is a multiple of 32, so the running column restarts at the same
    elements as in the register form."""
    K = 8
    for w in range(0, 401):
        nst = (w + K - 1) // K
        covered = []
        for t in range(nst):
            k0 = t * K
            kk = min(K, w - k0)
            covered += list(range(k0, k0 + kk))
            assert (k0 % CHUNK == 0) == any(k % CHUNK == 0 for k in range(k0, k0 + kk))
        assert covered == list(range(w))
