"""The row ranges of the persistent factor PCG, checked on the CPU.

Each CTA of the kernel computes z = M r for its rows [lo, hi) with
M = F^T F (FSAI, mode 2: the lower form F first) or M = F F^T (the learned
factor, mode 3: F^T first), F lower block-triangular on H's pattern. It
keeps r over a row range R and recomputes the first pass y over a row range
Y; no other rows are exchanged. The ranges follow the host layout rule:
* mode 2: Y = [lo, last column of the CTA's rows + 1); R = [first column of
  Y's rows, Y's end);
* mode 3: Y = [first column of the CTA's rows, hi); R = [Y's start, last
  column of Y's rows + 1);
both R ends widened to whole groups of 4 rows.

The test zeroes r outside R and y outside Y and checks that the CTA's rows
of z are unchanged, on a random factor over a mesh's real pattern.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from mfem_gb300 import beams


def block_pattern(mesh):
    t = mesh.tet_indices
    r = np.repeat(t, 4, axis=1).ravel()
    c = np.tile(t, (1, 4)).ravel()
    A = sp.csr_matrix((np.ones(r.size), (r, c)), shape=(mesh.n, mesh.n))
    A.sum_duplicates()
    A.sort_indices()
    return A.indptr, A.indices


def ranges(rp, ci, n, ctas, mode):
    cmin = np.array([ci[rp[j]:rp[j + 1]].min() for j in range(n)])
    cmax = np.array([ci[rp[j]:rp[j + 1]].max() for j in range(n)])
    out = []
    for c in range(ctas):
        lo, hi = n * c // ctas, n * (c + 1) // ctas
        wlo, whi = min(lo, cmin[lo:hi].min()), max(hi, cmax[lo:hi].max() + 1)
        if mode == 2:
            ylo, yhi = lo, whi
            rlo, rhi = min(ylo, cmin[ylo:yhi].min()), yhi
        else:
            ylo, yhi = wlo, hi
            rlo, rhi = ylo, max(yhi, cmax[ylo:yhi].max() + 1)
        rlo = min(rlo, lo) & ~3
        rhi = min((max(rhi, hi) + 3) & ~3, (n + 3) & ~3)
        out.append((lo, hi, ylo, yhi, rlo, rhi))
    return out


@pytest.mark.parametrize("mode", [2, 3])
@pytest.mark.parametrize("name,cells,ctas", [("nh_beam", (16, 4, 4), 7), ("cantilever", None, 3),
                                             ("stiff_beam", (12, 4, 4), 11)])
def test_two_hop_ranges_suffice(mode, name, cells, ctas):
    mesh = beams.build_beam(name, cells=cells)
    rp, ci = block_pattern(mesh)
    n = mesh.n
    rng = np.random.default_rng(3)
    # a random lower block-triangular F on H's lower pattern
    rows = np.repeat(np.arange(n), np.diff(rp))
    keep = ci <= rows
    blocks = rng.standard_normal((int(keep.sum()), 3, 3))
    F = sp.bsr_matrix((blocks, ci[keep], np.concatenate([[0], np.cumsum(np.bincount(rows[keep], minlength=n))])),
                      shape=(3 * n, 3 * n)).tocsr()
    F0, F1 = (F, F.T.tocsr()) if mode == 2 else (F.T.tocsr(), F)
    r = rng.standard_normal(3 * n)
    z_full = F1 @ (F0 @ r)
    for lo, hi, ylo, yhi, rlo, rhi in ranges(rp, ci, n, ctas, mode):
        r_cut = np.zeros_like(r)
        r_cut[3 * rlo:3 * min(rhi, n)] = r[3 * rlo:3 * min(rhi, n)]
        y = F0 @ r_cut
        y_cut = np.zeros_like(y)
        y_cut[3 * ylo:3 * yhi] = y[3 * ylo:3 * yhi]
        z = F1 @ y_cut
        np.testing.assert_allclose(z[3 * lo:3 * hi], z_full[3 * lo:3 * hi], rtol=1e-12, atol=1e-12)
        # both ranges cover the CTA's own rows (the kernel keeps them in R)
        assert rlo <= lo and rhi >= hi and ylo <= lo and yhi >= hi
