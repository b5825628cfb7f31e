// FP64 gate fuser with the reference's rules (src/simulator-mpi/fusion_mpi.hpp).
//
// Gates are queued as (matrix, diagonal flag, qubit ids). perform() composes
// them, in insertion order, into one dense 2^N x 2^N matrix over the sorted
// set of ids (bit l of the matrix index <-> l-th smallest id), the product
// later gates on the left. Controls that arrive with a gate while the queue is
// empty stay "global" controls of the fused gate; a control that is not shared
// by every queued gate is folded into the matrices as extra (highest) matrix
// bits, identity except the bottom-right block (fusion_mpi.hpp:167-226).
#pragma once
#include <complex>
#include <cstdint>
#include <set>
#include <algorithm>
#include <vector>

namespace hqs {

using cplx = std::complex<double>;

struct DenseGate {
    int dim = 0;                // rows (== cols), a power of two
    std::vector<cplx> m;        // row-major
    bool diag = false;
    std::vector<int64_t> ids;   // matrix bit j <-> ids[j]
};

// Fold ctrls into a gate as its highest matrix bits (fusion_mpi.hpp:167-187).
void add_controls(DenseGate& g, const std::vector<int64_t>& ctrls);

// Exact diagonality test on the unfolded matrix (funcs.hpp:325-337).
bool is_diagonal(const std::vector<cplx>& m, int dim);

// Sorted set of qubit ids in a flat vector (a fused gate holds at most a few).
struct IdSet {
    std::vector<int64_t> v;
    void insert(int64_t x) {
        auto it = std::lower_bound(v.begin(), v.end(), x);
        if (it == v.end() || *it != x) v.insert(it, x);
    }
    size_t count(int64_t x) const { return std::binary_search(v.begin(), v.end(), x) ? 1 : 0; }
    void erase(int64_t x) {
        auto it = std::lower_bound(v.begin(), v.end(), x);
        if (it != v.end() && *it == x) v.erase(it);
    }
    bool empty() const { return v.empty(); }
    size_t size() const { return v.size(); }
    void clear() { v.clear(); }
    std::vector<int64_t>::const_iterator begin() const { return v.begin(); }
    std::vector<int64_t>::const_iterator end() const { return v.end(); }
};

class Fusion {
public:
    // fusion_mpi.hpp:85-99: a 1x1 matrix only scales the fused gate.
    void insert(DenseGate g, const std::vector<int64_t>& ctrls);
    // fusion_mpi.hpp:101-165. Resets the scalar factor to 1 (like the reference)
    // but keeps the queued gates; callers clear() after a successful run.
    void perform(DenseGate& out, std::vector<int64_t>& ctrls);
    void clear();
    bool empty() const { return items_.empty(); }
    size_t num_qubits() const { return set_.size(); }
    size_t size() const { return items_.size(); }

private:
    void handle_controls(DenseGate& g, const std::vector<int64_t>& ctrls);

    IdSet set_;
    std::vector<DenseGate> items_;
    IdSet ctrl_set_;
    cplx factor_ = 1.0;
};

}  // namespace hqs
