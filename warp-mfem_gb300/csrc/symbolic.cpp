// Host-side symbolic analysis of the global system (run once per mesh).
//
// The reference rebuilds padded BSR topologies every Newton iteration with
// bsr_set_from_triplets and bsr_mm (src/mfem/refinement/solver.py:685-724),
// sized by a row capacity of 1 + 3 * max incident tets (solver.py:203).  The
// topology only changes with the mesh, so here it is computed once, exactly:
//
//  * the vertex-adjacency sparsity of H, diagonal included, ascending columns;
//  * the element -> slot map: the slot of block (tets[e][k], tets[e][l]);
//  * the same map inverted and sorted by slot (then by tet), which the
//    numeric assembly reduces with warp shuffles; whole slots are packed into
//    warp-sized chunks so no slot is split between warps.
#include <algorithm>
#include <cstring>

#include "internal.h"

namespace mfem {

static bool check_tets(int n, int T, const int32_t *tets, std::string &err) {
    if (n < 0 || T < 0) {
        err = "negative particle or tet count";
        return false;
    }
    if (T > 0 && tets == nullptr) {
        err = "tet_indices is NULL";
        return false;
    }
    if ((int64_t)T * 16 > (int64_t)INT32_MAX) {
        err = "too many tets for 32-bit contribution codes";
        return false;
    }
    for (int64_t i = 0; i < (int64_t)T * 4; ++i) {
        if (tets[i] < 0 || tets[i] >= n) {
            err = "tet_indices[" + std::to_string(i / 4) + "] references vertex " + std::to_string(tets[i]) +
                  " outside [0, " + std::to_string(n) + ")";
            return false;
        }
    }
    for (int e = 0; e < T; ++e) {
        const int32_t *t = tets + 4 * (int64_t)e;
        for (int a = 0; a < 4; ++a)
            for (int b = a + 1; b < 4; ++b)
                if (t[a] == t[b]) {
                    err = "tet " + std::to_string(e) + " repeats vertex " + std::to_string(t[a]);
                    return false;
                }
    }
    return true;
}

// Tets of each vertex, ascending, as codes tet * 4 + corner (a counting sort).
static void vertex_tets(int n, int T, const int32_t *tets, std::vector<int64_t> &vptr, std::vector<int32_t> &vcode) {
    vptr.assign((size_t)n + 1, 0);
    for (int64_t i = 0; i < (int64_t)T * 4; ++i) vptr[tets[i] + 1]++;
    for (int v = 0; v < n; ++v) vptr[v + 1] += vptr[v];
    vcode.assign((size_t)T * 4, 0);
    std::vector<int64_t> fill(vptr.begin(), vptr.end() - 1);
    for (int64_t i = 0; i < (int64_t)T * 4; ++i) vcode[fill[tets[i]]++] = (int32_t)i;
}

bool build_sparsity(int n, int T, const int32_t *tets, std::vector<int32_t> &row_ptr, std::vector<int32_t> &col_idx,
                    std::string &err) {
    if (!check_tets(n, T, tets, err)) return false;
    // per row: the diagonal and the vertices of the row's tets, made unique
    // with a stamp array and sorted (a few dozen columns a row)
    std::vector<int64_t> vptr;
    std::vector<int32_t> vcode;
    vertex_tets(n, T, tets, vptr, vcode);
    std::vector<int32_t> stamp((size_t)n, -1);
    std::vector<int32_t> row;
    row_ptr.assign((size_t)n + 1, 0);
    col_idx.clear();
    col_idx.reserve((size_t)T * 4 + (size_t)n);
    for (int v = 0; v < n; ++v) {
        row.clear();
        stamp[v] = v;
        row.push_back(v);
        for (int64_t i = vptr[v]; i < vptr[v + 1]; ++i) {
            const int32_t *t = tets + 4 * (int64_t)(vcode[i] >> 2);
            for (int l = 0; l < 4; ++l)
                if (stamp[t[l]] != v) {
                    stamp[t[l]] = v;
                    row.push_back(t[l]);
                }
        }
        std::sort(row.begin(), row.end());
        col_idx.insert(col_idx.end(), row.begin(), row.end());
        if (col_idx.size() > (size_t)INT32_MAX) {
            err = "sparsity exceeds 2^31 blocks";
            return false;
        }
        row_ptr[v + 1] = (int32_t)col_idx.size();
    }
    return true;
}

bool build_slot_map(int n, int T, const int32_t *tets, const int32_t *row_ptr, const int32_t *col_idx, int32_t *slots,
                    std::string &err) {
    if (!check_tets(n, T, tets, err)) return false;
    // per row: each column's slot through a stamped position array, then
    // the slots of the row's tet corners
    std::vector<int64_t> vptr;
    std::vector<int32_t> vcode;
    vertex_tets(n, T, tets, vptr, vcode);
    std::vector<int32_t> stamp((size_t)n, -1), pos((size_t)n, 0);
    for (int v = 0; v < n; ++v) {
        for (int32_t j = row_ptr[v]; j < row_ptr[v + 1]; ++j) {
            const int32_t c = col_idx[j];
            if (c < 0 || c >= n) {
                err = "column index out of range in row " + std::to_string(v);
                return false;
            }
            stamp[c] = v;
            pos[c] = j;
        }
        for (int64_t i = vptr[v]; i < vptr[v + 1]; ++i) {
            const int32_t e = vcode[i] >> 2, k = vcode[i] & 3;
            const int32_t *t = tets + 4 * (int64_t)e;
            for (int l = 0; l < 4; ++l) {
                if (stamp[t[l]] != v) {
                    err = "sparsity lacks block (" + std::to_string(v) + ", " + std::to_string(t[l]) + ")";
                    return false;
                }
                slots[(int64_t)e * 16 + k * 4 + l] = pos[t[l]];
            }
        }
    }
    return true;
}

bool build_tri_slots(int n, int n_tris, const int32_t *tris, const int32_t *row_ptr, const int32_t *col_idx,
                     int32_t *tri_slots, std::vector<int32_t> &vt_ptr, std::vector<int32_t> &vt_code,
                     std::string &err) {
    for (int t = 0; t < n_tris; ++t) {
        const int32_t *v = tris + 3 * (int64_t)t;
        for (int k = 0; k < 3; ++k) {
            if (v[k] < 0 || v[k] >= n) {
                err = "tri " + std::to_string(t) + " has a vertex index out of range";
                return false;
            }
        }
        if (v[0] == v[1] || v[1] == v[2] || v[0] == v[2]) {
            err = "tri " + std::to_string(t) + " repeats a vertex";
            return false;
        }
        for (int i = 0; i < 3; ++i) {
            const int32_t *b = col_idx + row_ptr[v[i]];
            const int32_t *e = col_idx + row_ptr[v[i] + 1];
            for (int j = 0; j < 3; ++j) {
                const int32_t *p = std::lower_bound(b, e, v[j]);
                if (p == e || *p != v[j]) {
                    err = "tri " + std::to_string(t) + " joins vertices that share no tet";
                    return false;
                }
                tri_slots[(int64_t)t * 9 + i * 3 + j] = (int32_t)(p - col_idx);
            }
        }
    }
    // incident tri corners of each vertex, in tri order
    vt_ptr.assign(n + 1, 0);
    for (int64_t i = 0; i < (int64_t)n_tris * 3; ++i) vt_ptr[tris[i] + 1]++;
    for (int v = 0; v < n; ++v) vt_ptr[v + 1] += vt_ptr[v];
    vt_code.assign((size_t)n_tris * 3, 0);
    std::vector<int32_t> fill(vt_ptr.begin(), vt_ptr.end() - 1);
    for (int64_t i = 0; i < (int64_t)n_tris * 3; ++i) vt_code[fill[tris[i]]++] = (int32_t)i;
    return true;
}

bool build_contributions(int n, int T, const int32_t *tets, const int32_t *row_ptr, const int32_t *slots,
                         Symbolic &sym, std::string &err, int n_tris, const int32_t *tri_slots) {
    (void)tets;
    const int64_t nnzb = row_ptr[n];
    if ((int64_t)T * 16 + (int64_t)n_tris * 9 > (int64_t)INT32_MAX) {
        err = "too many tets and tris for 32-bit contribution codes";
        return false;
    }
    std::vector<int32_t> count(nnzb + 1, 0);
    for (int64_t i = 0; i < (int64_t)T * 16; ++i) count[slots[i] + 1]++;
    for (int64_t i = 0; i < (int64_t)n_tris * 9; ++i) count[tri_slots[i] + 1]++;
    // a vertex without tets still owns its diagonal block (mass + attachment):
    // give it one empty contribution so the assembly visits it
    std::vector<int32_t> isolated;  // vertices in no tet
    std::vector<int32_t> isolated_slot;
    for (int v = 0; v < n; ++v) {
        const int32_t *b = sym.col_idx.data() + row_ptr[v];
        const int32_t *e = sym.col_idx.data() + row_ptr[v + 1];
        const int32_t *p = std::lower_bound(b, e, v);
        if (p == e || *p != v) {
            err = "sparsity lacks diagonal block of vertex " + std::to_string(v);
            return false;
        }
        const int32_t ds = (int32_t)(p - sym.col_idx.data());
        if (count[ds + 1] == 0) {
            count[ds + 1] = 1;
            isolated.push_back(v);
            isolated_slot.push_back(ds);
        }
    }
    std::vector<int64_t> start(nnzb + 1, 0);
    for (int64_t s = 0; s < nnzb; ++s) start[s + 1] = start[s] + count[s + 1];
    const int64_t total = start[nnzb];
    if (total > (int64_t)INT32_MAX) {
        err = "too many contributions";
        return false;
    }
    sym.contrib_code.assign(total, 0);
    sym.contrib_slot.assign(total, 0);
    std::vector<int64_t> fill(start.begin(), start.end() - 1);
    for (size_t i = 0; i < isolated.size(); ++i) {
        const int32_t s = isolated_slot[i];
        sym.contrib_code[fill[s]] = -(isolated[i] + 1);
        sym.contrib_slot[fill[s]] = s;
        fill[s]++;
    }
    for (int e = 0; e < T; ++e)
        for (int kl = 0; kl < 16; ++kl) {
            const int32_t s = slots[(int64_t)e * 16 + kl];
            const int64_t pos = fill[s]++;
            sym.contrib_code[pos] = e * 16 + kl;
            sym.contrib_slot[pos] = s;
        }
    // surface-tri contact blocks (i, j) after the tets of their slot, coded
    // 16 T + 9 tri + 3 i + j
    for (int t = 0; t < n_tris; ++t)
        for (int ij = 0; ij < 9; ++ij) {
            const int32_t s = tri_slots[(int64_t)t * 9 + ij];
            const int64_t pos = fill[s]++;
            sym.contrib_code[pos] = 16 * T + 9 * t + ij;
            sym.contrib_slot[pos] = s;
        }
    // pack whole slots into chunks of <= 32 contributions (a longer slot gets
    // a chunk of its own)
    sym.chunk_ptr.clear();
    sym.chunk_ptr.push_back(0);
    int64_t chunk_len = 0;
    for (int64_t s = 0; s < nnzb; ++s) {
        const int64_t len = start[s + 1] - start[s];
        if (len == 0) continue;
        if (chunk_len > 0 && chunk_len + len > 32) {
            sym.chunk_ptr.push_back((int32_t)start[s]);
            chunk_len = 0;
        }
        chunk_len += len;
        if (chunk_len >= 32) {
            sym.chunk_ptr.push_back((int32_t)start[s + 1]);
            chunk_len = 0;
        }
    }
    if (chunk_len > 0) sym.chunk_ptr.push_back((int32_t)total);
    return true;
}

}  // namespace mfem
