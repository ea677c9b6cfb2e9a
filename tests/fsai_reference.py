"""Float64 numpy FSAI on a BSR block pattern: the reference the FSAI tests
compare the device factor against (tests/test_fsai_reference.py checks it on
CPU).  Block row i over the row's lower columns P: G[i, P] = the last block
row of chol(H[P, P])^-1, in the order of the lower pattern (columns <= row,
ascending)."""
import numpy as np


def lower_pattern(rp, ci):
    """Row pointers, columns and H-slot of each block of the lower block
    pattern (columns <= row, ascending)."""
    n = len(rp) - 1
    lrow, lcol, lslot = [0], [], []
    for r in range(n):
        for k in range(rp[r], rp[r + 1]):
            if ci[k] <= r:
                lcol.append(ci[k])
                lslot.append(k)
        lrow.append(len(lcol))
    return np.array(lrow), np.array(lcol), np.array(lslot)


def fsai_numpy(rp, ci, vals, max_cols=16):
    """Float64 block FSAI [nnzl, 3, 3] on the lower block pattern; rows with
    more than max_cols lower blocks are listed (the kernel falls back)."""
    lrow, lcol, _ = lower_pattern(rp, ci)
    n = len(rp) - 1
    G = np.zeros((len(lcol), 3, 3))
    slot = {}
    for r in range(n):
        for k in range(rp[r], rp[r + 1]):
            slot[(r, ci[k])] = k
    fallback = []
    for i in range(n):
        P = lcol[lrow[i]:lrow[i + 1]]
        if len(P) > max_cols:
            fallback.append(i)
            continue
        m = len(P)
        A = np.zeros((3 * m, 3 * m))
        for a, pa in enumerate(P):
            for b, pb in enumerate(P):
                k = slot.get((pa, pb))
                if k is not None:
                    A[3 * a:3 * a + 3, 3 * b:3 * b + 3] = vals[k]
        Linv = np.linalg.inv(np.linalg.cholesky(A))
        Gi = Linv[-3:, :]
        for a in range(m):
            G[lrow[i] + a] = Gi[:, 3 * a:3 * a + 3]
    return G, fallback
