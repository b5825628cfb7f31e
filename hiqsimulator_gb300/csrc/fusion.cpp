#include "fusion.h"

#include <algorithm>

namespace hqs {

void add_controls(DenseGate& g, const std::vector<int64_t>& ctrls) {
    if (ctrls.empty()) return;
    const int F = 1 << ctrls.size();
    const int nd = F * g.dim;
    std::vector<cplx> nm((size_t)nd * nd, cplx(0.0, 0.0));
    const int off = nd - g.dim;
    for (int i = 0; i < off; ++i) nm[(size_t)i * nd + i] = 1.0;
    for (int i = 0; i < g.dim; ++i)
        for (int j = 0; j < g.dim; ++j) nm[(size_t)(off + i) * nd + off + j] = g.m[(size_t)i * g.dim + j];
    g.m.swap(nm);
    g.dim = nd;
    g.ids.insert(g.ids.end(), ctrls.begin(), ctrls.end());
}

bool is_diagonal(const std::vector<cplx>& m, int dim) {
    for (int i = 0; i < dim; ++i)
        for (int j = 0; j < dim; ++j)
            if (i != j && m[(size_t)i * dim + j] != cplx(0.0, 0.0)) return false;
    return true;
}

void Fusion::insert(DenseGate g, const std::vector<int64_t>& ctrls) {
    if (g.dim == 1) {
        factor_ *= g.m[0];
        return;
    }
    for (int64_t id : g.ids) set_.insert(id);
    handle_controls(g, ctrls);
    items_.push_back(std::move(g));
}

void Fusion::handle_controls(DenseGate& g, const std::vector<int64_t>& ctrls) {
    if (ctrls.empty() && ctrl_set_.empty()) return;
    IdSet unhandled = ctrl_set_;
    for (int64_t c : ctrls) {
        if (ctrl_set_.count(c) == 0) {
            if (!items_.empty()) {
                add_controls(g, {c});
                set_.insert(c);
            } else {
                ctrl_set_.insert(c);
            }
        } else {
            unhandled.erase(c);
        }
    }
    if (!unhandled.empty()) {
        std::vector<int64_t> moved(unhandled.begin(), unhandled.end());
        for (int64_t c : moved) {
            ctrl_set_.erase(c);
            set_.insert(c);
        }
        for (auto& it : items_) add_controls(it, moved);
    }
}

void Fusion::perform(DenseGate& out, std::vector<int64_t>& ctrls) {
    out.ids.assign(set_.begin(), set_.end());
    const int N = (int)out.ids.size();
    const int dim = 1 << N;
    out.dim = dim;
    out.m.assign((size_t)dim * dim, cplx(0.0, 0.0));
    for (int i = 0; i < dim; ++i) out.m[(size_t)i * dim + i] = factor_;
    out.diag = true;
    for (const auto& it : items_) {
        if (!it.diag) out.diag = false;
        const int k = (int)it.ids.size();
        const int D = 1 << k;
        // off[j]: the fused-matrix row offset of item row / column j; x: the
        // gathered rows (on the stack up to 5 qubits, the largest a pass runs)
        constexpr int kStack = 32;
        uint32_t off_s[kStack];
        cplx x_s[kStack];
        std::vector<uint32_t> off_h;
        std::vector<cplx> x_h;
        uint32_t* off = off_s;
        cplx* x = x_s;
        if (D > kStack) {
            off_h.resize(D);
            x_h.resize(D);
            off = off_h.data();
            x = x_h.data();
        }
        for (int j = 0; j < D; ++j) off[j] = 0;
        uint32_t itmask = 0;
        for (int l = 0; l < k; ++l) {
            const uint32_t b = 1u << (std::lower_bound(out.ids.begin(), out.ids.end(), it.ids[l]) - out.ids.begin());
            itmask |= b;
            for (int j = 0; j < D; ++j)
                if ((j >> l) & 1) off[j] |= b;
        }
        // new M[:, c] = (item (x) I) old M[:, c]: per column, each group of D
        // rows that differ only in the item's bits is gathered, multiplied by
        // the item and written back (the same products, summed in the same
        // order, as row by row)
        for (int c = 0; c < dim; ++c)
            for (uint32_t base = 0; base < (uint32_t)dim; ++base) {
                if (base & itmask) continue;
                for (int j = 0; j < D; ++j) x[j] = out.m[(size_t)(base | off[j]) * dim + c];
                for (int jo = 0; jo < D; ++jo) {
                    cplx acc(0.0, 0.0);
                    for (int j = 0; j < D; ++j) acc += x[j] * it.m[(size_t)jo * it.dim + j];
                    out.m[(size_t)(base | off[jo]) * dim + c] = acc;
                }
            }
    }
    ctrls.assign(ctrl_set_.begin(), ctrl_set_.end());
    factor_ = 1.0;
}

void Fusion::clear() {
    set_.clear();
    items_.clear();
    ctrl_set_.clear();
    factor_ = 1.0;
}

}  // namespace hqs
