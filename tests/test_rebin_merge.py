"""The arithmetic of ULMPM's re-binning update (karamelo_gb300/csrc/kmpm_rebin.cu)
restated in numpy and checked against a stable sort (CPU).

The kernels place the particle of slot i and new cell k at
    cs[k] + clamp(stayers before i - stayers with cell < k, 0, stayers in k)
          + (movers into k with slot < i),
with the new cell starts cs from the old per-cell counts minus the movers
out plus the movers in.  These tests check that formula, and the new ranges,
against numpy's stable argsort of the new keys: random cells, near-sorted
inputs where a fraction of particles moves a few cells, and the start state
(every slot in cell 0).  tests/test_gpu_rebin.py checks the CUDA kernels
against the full radix sort on the GPU.
"""
import numpy as np
import pytest


def rebin(keys, cs, ce, knew, ncell):
    """keys: sorted keys of the current slots; cs/ce: their cell ranges;
    knew: the new key of every slot.  Returns (perm, sorted keys, new cs,
    new ce) as the kernels form them."""
    n = len(keys)
    mover = knew != keys
    cin = np.bincount(knew[mover], minlength=ncell)
    cout = np.bincount(keys[mover], minlength=ncell)
    newcnt = (ce - cs) - cout + cin                       # k_rebin_count / ranges
    csn = np.concatenate([[0], np.cumsum(newcnt)])[:ncell]
    cen = csn + newcnt
    mpre = np.concatenate([[0], np.cumsum(cin)])          # movers' prefix (ncell + 1)
    movers = np.nonzero(mover)[0]
    bsort = np.zeros(len(movers), np.int64)               # k_rebin_group / order
    for k in np.unique(knew[movers]):
        bsort[mpre[k]:mpre[k + 1]] = np.sort(movers[knew[movers] == k])
    before = np.concatenate([[0], np.cumsum(mover)])[:n]  # movers before slot i (blkm scan)
    perm = np.full(n, -1)
    out = np.full(n, -1)
    for i in range(n):                                    # k_rebin_place
        k = knew[i]
        csk, cnt = csn[k], cen[k] - csn[k]
        mp, mc = mpre[k], mpre[k + 1] - mpre[k]
        a = min(max((i - before[i]) - (csk - mp), 0), cnt - mc)
        b = int(np.sum(bsort[mp:mp + mc] < i))
        pos = csk + a + b
        assert perm[pos] == -1, "two slots at one destination"
        perm[pos] = i
        out[pos] = k
    return perm, out, csn, cen


def ranges_of(sorted_keys, ncell):
    return (np.searchsorted(sorted_keys, np.arange(ncell), "left"),
            np.searchsorted(sorted_keys, np.arange(ncell), "right"))


def check(keys, cs, ce, knew, ncell):
    perm, out, csn, cen = rebin(keys, cs, ce, knew, ncell)
    ref = np.argsort(knew, kind="stable")
    assert np.array_equal(perm, ref)
    assert np.array_equal(out, knew[ref])
    rs, re = ranges_of(knew[ref], ncell)
    assert np.array_equal(csn, rs) and np.array_equal(cen, re)


@pytest.mark.parametrize("seed", range(40))
def test_near_sorted_update_is_the_stable_sort(seed):
    rng = np.random.default_rng(seed)
    ncell = int(rng.integers(1, 80))
    n = int(rng.integers(1, 500))
    keys = np.sort(rng.integers(0, ncell, n))
    cs, ce = ranges_of(keys, ncell)
    knew = keys.copy()
    m = rng.random(n) < rng.random() * 0.6
    knew[m] = np.clip(keys[m] + rng.integers(-3, 4, m.sum()), 0, ncell - 1)
    check(keys, cs, ce, knew, ncell)


@pytest.mark.parametrize("seed", range(20))
def test_start_state_every_slot_in_cell_zero(seed):
    """The binning the first step updates: keys all 0, cell 0 holds every slot."""
    rng = np.random.default_rng(100 + seed)
    ncell = int(rng.integers(1, 60))
    n = int(rng.integers(1, 400))
    keys = np.zeros(n, np.int64)
    cs, ce = np.zeros(ncell, np.int64), np.zeros(ncell, np.int64)
    ce[0] = n
    check(keys, cs, ce, rng.integers(0, ncell, n), ncell)


def test_no_movers_and_all_movers():
    keys = np.repeat(np.arange(10), 3)
    cs, ce = ranges_of(keys, 12)
    check(keys, cs, ce, keys.copy(), 12)                      # nothing moves: identity
    check(keys, cs, ce, (keys + 1) % 12, 12)                  # every particle moves
    check(keys, cs, ce, np.full_like(keys, 11), 12)           # all into one cell
