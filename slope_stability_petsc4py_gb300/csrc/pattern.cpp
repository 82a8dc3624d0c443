// Host builder of the fixed owned-row CSR pattern and the element->CSR maps.
//
// Produces exactly what prepare_owned_tangent_pattern builds with dictionary loops
// (src/slope_stability/fem/distributed_tangent.py):
//   overlap partition        distributed_elastic.py:36-52 (elements touching owned nodes,
//                            sorted unique overlap nodes)
//   element dof lids         distributed_tangent.py:993-999
//   structural CSR           distributed_tangent.py:440-478 (free rows: sorted union of the free
//                            columns of every overlap element holding the row's node; constrained
//                            rows: only the diagonal)
//   constrained diagonals    distributed_tangent.py:297-325
//   scatter map              distributed_tangent.py:328-366 ([e][a*n_ld+b] -> CSR position or -1)
//   row slots                distributed_tangent.py:369-437 (slots grouped by row, filled in
//                            element order then local-dof order)
// plus elem_row ([e][a] -> owned free row or -1) used by the element force kernel.
//
// The column set of a free row depends only on its node (every component of a node sees the
// same incident elements), so columns are gathered once per owned node and positions are found
// by binary search in the node's sorted column list.
#include <algorithm>
#include <climits>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ssp_gb300.h"

struct ssp_pattern {
    int dim = 0, n_p = 0, n_ld = 0;
    int64_t n_rows = 0;
    std::vector<int64_t> overlap_elements, overlap_nodes, owned_local_overlap_dofs;
    std::vector<int32_t> dof_lids, indptr, indices, cdiag, scatter, row_slot_ptr, slot_elem, slot_pos, elem_row;
    std::vector<uint8_t> slot_lrow, owned_free;
};

template <typename T>
static int copy_out(const std::vector<T> &v, void *dst) {
    if (!v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(T));
    return SSP_OK;
}

extern "C" {

int ssp_pattern_build(int dim, int n_nodes, int n_p, int n_elem, const int64_t *elem, const uint8_t *free_mask,
                      int node0, int node1, ssp_pattern **out) {
    if (!out || (dim != 2 && dim != 3) || n_nodes < 0 || n_p <= 0 || n_elem < 0 || node0 < 0 || node1 < node0 ||
        node1 > n_nodes || (n_elem > 0 && !elem) || (n_nodes > 0 && !free_mask))
        return SSP_ERR_INVALID;
    const int n_ld = dim * n_p;
    if (n_ld > 255) return SSP_ERR_OVERFLOW;  // slot_lrow is uint8 (distributed_tangent.py:383-384)
    auto *P = new ssp_pattern();
    P->dim = dim;
    P->n_p = n_p;
    P->n_ld = n_ld;
    const int64_t row0 = (int64_t)dim * node0, row1 = (int64_t)dim * node1;
    const int64_t n_rows = row1 - row0;
    P->n_rows = n_rows;
    auto node_of = [&](int a, int64_t e) { return elem[(int64_t)a * n_elem + e]; };

    // overlap elements and nodes
    for (int64_t e = 0; e < n_elem; ++e) {
        for (int a = 0; a < n_p; ++a) {
            const int64_t nd = node_of(a, e);
            if (nd < 0 || nd >= n_nodes) {
                delete P;
                return SSP_ERR_INVALID;
            }
            if (nd >= node0 && nd < node1) {
                P->overlap_elements.push_back(e);
                break;
            }
        }
    }
    const int64_t n_ov = (int64_t)P->overlap_elements.size();
    {
        std::vector<uint8_t> seen(n_nodes, 0);
        for (int64_t k = 0; k < n_ov; ++k)
            for (int a = 0; a < n_p; ++a) seen[node_of(a, P->overlap_elements[k])] = 1;
        for (int64_t nd = 0; nd < n_nodes; ++nd)
            if (seen[nd]) P->overlap_nodes.push_back(nd);
    }
    std::vector<int64_t> lid(n_nodes, -1);
    for (size_t i = 0; i < P->overlap_nodes.size(); ++i) lid[P->overlap_nodes[i]] = (int64_t)i;
    for (int64_t nd = node0; nd < node1; ++nd) {
        if (lid[nd] < 0) {  // owned node outside the overlap submesh (distributed_elastic.py:138-139)
            delete P;
            return SSP_ERR_PATTERN;
        }
    }
    if ((int64_t)P->overlap_nodes.size() * dim > INT32_MAX) {
        delete P;
        return SSP_ERR_OVERFLOW;
    }
    P->dof_lids.resize(n_ov * n_ld);
    for (int64_t k = 0; k < n_ov; ++k)
        for (int a = 0; a < n_p; ++a)
            for (int c = 0; c < dim; ++c)
                P->dof_lids[k * n_ld + a * dim + c] = (int32_t)(dim * lid[node_of(a, P->overlap_elements[k])] + c);
    P->owned_local_overlap_dofs.resize(n_rows);
    for (int64_t nd = node0; nd < node1; ++nd)
        for (int c = 0; c < dim; ++c) P->owned_local_overlap_dofs[(nd - node0) * dim + c] = dim * lid[nd] + c;
    P->owned_free.resize(n_rows);
    for (int64_t r = 0; r < n_rows; ++r) P->owned_free[r] = free_mask[row0 + r] ? 1 : 0;

    // per owned node: sorted free columns of all incident overlap elements
    const int64_t n_own_nodes = node1 - node0;
    std::vector<std::vector<int32_t>> node_cols(n_own_nodes);
    {
        std::vector<int64_t> deg(n_own_nodes + 1, 0);
        for (int64_t k = 0; k < n_ov; ++k)
            for (int a = 0; a < n_p; ++a) {
                const int64_t nd = node_of(a, P->overlap_elements[k]);
                if (nd >= node0 && nd < node1) deg[nd - node0 + 1]++;
            }
        for (int64_t i = 0; i < n_own_nodes; ++i) deg[i + 1] += deg[i];
        std::vector<int64_t> inc(deg[n_own_nodes]);
        std::vector<int64_t> fill(deg.begin(), deg.end() - 1);
        for (int64_t k = 0; k < n_ov; ++k)
            for (int a = 0; a < n_p; ++a) {
                const int64_t nd = node_of(a, P->overlap_elements[k]);
                if (nd >= node0 && nd < node1) inc[fill[nd - node0]++] = k;
            }
        for (int64_t i = 0; i < n_own_nodes; ++i) {
            std::vector<int32_t> &cols = node_cols[i];
            for (int64_t t = deg[i]; t < deg[i + 1]; ++t) {
                const int64_t e = P->overlap_elements[inc[t]];
                for (int b = 0; b < n_p; ++b) {
                    const int64_t nb = node_of(b, e);
                    for (int c = 0; c < dim; ++c) {
                        const int64_t col = dim * nb + c;
                        if (free_mask[col]) {
                            if (col > INT32_MAX) {
                                delete P;
                                return SSP_ERR_OVERFLOW;
                            }
                            cols.push_back((int32_t)col);
                        }
                    }
                }
            }
            std::sort(cols.begin(), cols.end());
            cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
        }
    }

    // CSR
    P->indptr.assign(n_rows + 1, 0);
    int64_t nnz = 0;
    for (int64_t r = 0; r < n_rows; ++r) {
        nnz += P->owned_free[r] ? (int64_t)node_cols[r / dim].size() : 1;
        if (nnz > INT32_MAX) {
            delete P;
            return SSP_ERR_OVERFLOW;
        }
        P->indptr[r + 1] = (int32_t)nnz;
    }
    P->indices.resize(nnz);
    for (int64_t r = 0; r < n_rows; ++r) {
        if (P->owned_free[r]) {
            const auto &cols = node_cols[r / dim];
            std::copy(cols.begin(), cols.end(), P->indices.begin() + P->indptr[r]);
        } else {
            P->indices[P->indptr[r]] = (int32_t)(row0 + r);
            P->cdiag.push_back(P->indptr[r]);
        }
    }

    // scatter map, elem_row, slot counts
    const int64_t n_map = n_ov * (int64_t)n_ld * n_ld;
    P->scatter.assign(n_map, -1);
    P->elem_row.assign(n_ov * n_ld, -1);
    std::vector<int64_t> counts(n_rows, 0);
    std::vector<int64_t> gdof(n_ld);
    for (int64_t k = 0; k < n_ov; ++k) {
        const int64_t e = P->overlap_elements[k];
        for (int a = 0; a < n_p; ++a)
            for (int c = 0; c < dim; ++c) gdof[a * dim + c] = dim * node_of(a, e) + c;
        for (int a = 0; a < n_ld; ++a) {
            const int64_t R = gdof[a];
            if (R < row0 || R >= row1 || !P->owned_free[R - row0]) continue;
            const int64_t lr = R - row0;
            P->elem_row[k * n_ld + a] = (int32_t)lr;
            counts[lr]++;
            const auto &cols = node_cols[lr / dim];
            int32_t *dst = &P->scatter[(k * n_ld + a) * n_ld];
            for (int b = 0; b < n_ld; ++b) {
                const int64_t C = gdof[b];
                if (!free_mask[C]) continue;
                auto it = std::lower_bound(cols.begin(), cols.end(), (int32_t)C);
                if (it == cols.end() || *it != (int32_t)C) {
                    delete P;
                    return SSP_ERR_PATTERN;
                }
                dst[b] = P->indptr[lr] + (int32_t)(it - cols.begin());
            }
        }
    }

    // row slots
    P->row_slot_ptr.assign(n_rows + 1, 0);
    int64_t n_slots = 0;
    for (int64_t r = 0; r < n_rows; ++r) {
        n_slots += counts[r];
        if (n_slots > INT32_MAX) {
            delete P;
            return SSP_ERR_OVERFLOW;
        }
        P->row_slot_ptr[r + 1] = (int32_t)n_slots;
    }
    P->slot_elem.resize(n_slots);
    P->slot_lrow.resize(n_slots);
    P->slot_pos.resize(n_slots * n_ld);
    std::vector<int64_t> wp(P->row_slot_ptr.begin(), P->row_slot_ptr.end() - 1);
    for (int64_t k = 0; k < n_ov; ++k) {
        for (int a = 0; a < n_ld; ++a) {
            const int32_t lr = P->elem_row[k * n_ld + a];
            if (lr < 0) continue;
            const int64_t s = wp[lr]++;
            P->slot_elem[s] = (int32_t)k;
            P->slot_lrow[s] = (uint8_t)a;
            std::memcpy(&P->slot_pos[s * n_ld], &P->scatter[(k * n_ld + a) * n_ld], sizeof(int32_t) * n_ld);
        }
    }
    *out = P;
    return SSP_OK;
}

int ssp_pattern_sizes(const ssp_pattern *p, int64_t *sizes) {
    if (!p || !sizes) return SSP_ERR_INVALID;
    sizes[0] = (int64_t)p->overlap_elements.size();
    sizes[1] = (int64_t)p->overlap_nodes.size();
    sizes[2] = p->n_rows;
    sizes[3] = (int64_t)p->indices.size();
    sizes[4] = (int64_t)p->slot_elem.size();
    sizes[5] = (int64_t)p->cdiag.size();
    sizes[6] = p->n_ld;
    return SSP_OK;
}

int ssp_pattern_copy(const ssp_pattern *p, const char *name, void *dst) {
    if (!p || !name || !dst) return SSP_ERR_INVALID;
    const std::string n(name);
    if (n == "overlap_elements") return copy_out(p->overlap_elements, dst);
    if (n == "overlap_nodes") return copy_out(p->overlap_nodes, dst);
    if (n == "overlap_element_dof_lids") return copy_out(p->dof_lids, dst);
    if (n == "owned_local_overlap_dofs") return copy_out(p->owned_local_overlap_dofs, dst);
    if (n == "indptr") return copy_out(p->indptr, dst);
    if (n == "indices") return copy_out(p->indices, dst);
    if (n == "constrained_diag_positions") return copy_out(p->cdiag, dst);
    if (n == "scatter_map") return copy_out(p->scatter, dst);
    if (n == "row_slot_ptr") return copy_out(p->row_slot_ptr, dst);
    if (n == "slot_elem") return copy_out(p->slot_elem, dst);
    if (n == "slot_lrow") return copy_out(p->slot_lrow, dst);
    if (n == "slot_pos") return copy_out(p->slot_pos, dst);
    if (n == "elem_row") return copy_out(p->elem_row, dst);
    if (n == "owned_free_mask") return copy_out(p->owned_free, dst);
    return SSP_ERR_INVALID;
}

void ssp_pattern_free(ssp_pattern *p) { delete p; }

}  // extern "C"
