"""The index argument behind the early BWT of the host path, on the CPU.

The BWT row of SA slot s lands at U[s + 1] before the primary row i0 (the slot
of suffix 0) and at U[s] after it; U[0] = T[n - 1].  An early BWT is taken
while suffix 0 may still sit anywhere in its group's slot range [gs, ge), with
a provisional i0' from that range; the rows of every still-unresolved slot --
a superset of [gs, ge) -- are rewritten later with the final i0.  This checks,
on random permutations, that every U position is then right."""
import numpy as np


def bwt_rows(sa, T, i0, rows):
    """{U index: symbol} of the given SA rows under primary row i0."""
    n = len(T)
    out = {}
    for s in rows:
        if s == i0:
            continue
        k = s + 1 if s < i0 else s
        out[k] = T[sa[s] - 1]
    return out


def test_provisional_primary_row_is_repaired():
    rng = np.random.default_rng(5)
    for _ in range(300):
        n = int(rng.integers(3, 60))
        T = rng.integers(0, 4, n)
        sa = rng.permutation(n)
        i0 = int(np.nonzero(sa == 0)[0][0])
        gs = int(rng.integers(0, i0 + 1))
        ge = int(rng.integers(i0 + 1, n + 1))
        i0p = int(rng.integers(gs, ge))                    # provisional slot of suffix 0
        unresolved = set(range(gs, ge)) | set(int(x) for x in rng.integers(0, n, int(rng.integers(0, 4))))
        # early BWT: every row, provisional i0 (unresolved rows hold anything: here a wrong suffix)
        early_sa = sa.copy()
        for s in unresolved:
            early_sa[s] = int(rng.integers(1, n)) if n > 1 else 1
        early_sa[i0p], early_sa[i0] = 0, early_sa[i0p] if i0p != i0 else 0
        U = np.full(n, -1)
        U[0] = T[n - 1]
        for k, v in bwt_rows(early_sa, T, i0p, [s for s in range(n)]).items():
            U[k] = v
        # patch: the unresolved rows with the final SA and primary row
        for k, v in bwt_rows(sa, T, i0, sorted(unresolved)).items():
            U[k] = v
        final = np.full(n, -1)
        final[0] = T[n - 1]
        for k, v in bwt_rows(sa, T, i0, range(n)).items():
            final[k] = v
        assert np.array_equal(U, final), (n, gs, ge, i0, i0p)


def test_patch_covers_every_late_slot():
    """The SA patch writes the marked slots in address order, a warp per 32
    slots: every marked slot, nothing else."""
    rng = np.random.default_rng(6)
    for _ in range(50):
        n = int(rng.integers(1, 5000))
        marked = np.unique(rng.integers(0, n, int(rng.integers(0, n))))
        bits = np.zeros((n + 31) // 32, dtype=np.uint32)
        for s in marked:
            bits[s >> 5] |= np.uint32(1 << (s & 31))
        written = []
        for base in range(0, len(bits), 32):                 # one warp: 32 words
            for w in range(base, min(base + 32, len(bits))):
                m = int(bits[w])
                for lane in range(32):
                    s = w * 32 + lane
                    if (m >> lane) & 1 and s < n:
                        written.append(s)
        assert written == sorted(int(x) for x in marked)
