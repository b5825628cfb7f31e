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
    std::set<int64_t> unhandled = ctrl_set_;
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
    std::vector<cplx> col(dim);
    for (const auto& it : items_) {
        if (!it.diag) out.diag = false;
        const int k = (int)it.ids.size();
        std::vector<int> bit(k);
        for (int l = 0; l < k; ++l)
            bit[l] = (int)(std::lower_bound(out.ids.begin(), out.ids.end(), it.ids[l]) - out.ids.begin());
        uint32_t itmask = 0;
        for (int l = 0; l < k; ++l) itmask |= 1u << bit[l];
        // local index of every row of the fused matrix within the item
        std::vector<int> loc(dim);
        for (int i = 0; i < dim; ++i) {
            int li = 0;
            for (int l = 0; l < k; ++l) li |= ((i >> bit[l]) & 1) << l;
            loc[i] = li;
        }
        std::vector<int> scatter(1 << k);
        // new M[:, c] = (item (x) I) old M[:, c]
        for (int c = 0; c < dim; ++c) {
            for (int i = 0; i < dim; ++i) col[i] = out.m[(size_t)i * dim + c];
            for (int i = 0; i < dim; ++i) {
                const int li = loc[i];
                const uint32_t base = (uint32_t)i & ~itmask;
                cplx acc(0.0, 0.0);
                for (int j = 0; j < (1 << k); ++j) {
                    uint32_t src = base;
                    for (int l = 0; l < k; ++l)
                        if ((j >> l) & 1) src |= 1u << bit[l];
                    acc += col[src] * it.m[(size_t)li * it.dim + j];
                }
                out.m[(size_t)i * dim + c] = acc;
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
