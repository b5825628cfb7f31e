// Greedy gate clustering ("greedy fusion k <= K") on the host.
//
// Same rule as HiQ's GreedyScheduler driving ClusterScheduler
// (hiq/projectq/cengines/_greedyscheduler.py:119-137,
// src/scheduler/cluster_scheduler.{h,cpp}): among all sets C of at most K
// local qubits, reachable by growing the local qubits of some gate with
// higher-numbered qubits, pick the one that lets the most gates run in order
// (a gate runs when all its qubits are in C and none was touched by an
// earlier gate that could not run); ties go to fewer qubits, then to the set
// met first in that growth order. Emit the chosen gates as one cluster, drop
// them, repeat. Every gate counts as non-diagonal (_greedyscheduler.py:28).
// The choice and its tie-break order are kept exactly so that the fused
// matrices equal those of the reference pipeline.
#include <algorithm>
#include <cstdint>
#include <unordered_map>
#include <vector>

namespace hqs {

namespace {

struct Chooser {
    int K = 0;
    const std::vector<uint64_t>* gate = nullptr;  // all qubits (targets | controls) per gate
    const std::vector<uint64_t>* tgt = nullptr;
    uint64_t locals = 0, all = 0;
    int best = 0;
    uint64_t best_set = 0;
    std::unordered_map<uint64_t, uint64_t> tried;  // set -> growth bits already tried

    bool takeable(size_t i, uint64_t set, uint64_t blocked) const {
        const uint64_t q = (*gate)[i];
        if ((q & blocked) || ((q & locals) & ~set)) return false;
        return ((*tgt)[i] & ~locals) == 0;
    }
    int count(uint64_t set) const {
        uint64_t blocked = 0;
        int c = 0;
        for (size_t i = 0; i < gate->size(); ++i) {
            if (takeable(i, set, blocked)) {
                ++c;
            } else {
                blocked |= (*gate)[i];
                if ((blocked & all) == all) break;
            }
        }
        return c;
    }
    void consider(uint64_t set) {
        auto it = tried.find(set);
        if (it != tried.end() && it->second != 0) return;
        const int c = count(set);
        if (c > best || (c == best && __builtin_popcountll(set) < __builtin_popcountll(best_set))) {
            best = c;
            best_set = set;
        }
    }
    void grow(uint64_t set, uint64_t bit) {
        consider(set);
        if (bit > locals) return;
        uint64_t& t = tried[set];
        if (t & bit) return;
        t |= bit;
        if (!(bit & ~locals) && !(bit & set) && __builtin_popcountll(set) < K) grow(set | bit, bit << 1);
        grow(set, bit << 1);
    }
};

}  // namespace

// Returns the number of clusters, or -1 when 64 or more distinct qubits occur.
int greedy_schedule(int ngates, const int64_t* tgt, const int* toff, const int64_t* ctl, const int* coff, int nlocals,
                    const int64_t* locals, int K, int* order, int* cluster_end) {
    std::vector<int64_t> ids(locals, locals + nlocals);
    ids.insert(ids.end(), tgt, tgt + toff[ngates]);
    ids.insert(ids.end(), ctl, ctl + coff[ngates]);
    std::sort(ids.begin(), ids.end());
    ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
    if (ids.size() >= 64) return -1;
    auto bit_of = [&](int64_t id) {
        return 1ULL << (std::lower_bound(ids.begin(), ids.end(), id) - ids.begin());
    };
    uint64_t locm = 0;
    for (int i = 0; i < nlocals; ++i) locm |= bit_of(locals[i]);
    std::vector<uint64_t> gt(ngates), ga(ngates);
    for (int g = 0; g < ngates; ++g) {
        uint64_t t = 0, c = 0;
        for (int j = toff[g]; j < toff[g + 1]; ++j) t |= bit_of(tgt[j]);
        for (int j = coff[g]; j < coff[g + 1]; ++j) c |= bit_of(ctl[j]);
        gt[g] = t;
        ga[g] = t | c;
    }
    std::vector<int> live(ngates);
    for (int g = 0; g < ngates; ++g) live[g] = g;
    int emitted = 0, nclusters = 0;
    std::vector<uint64_t> rt, ra;
    while (!live.empty()) {
        // Bit positions are the ranks of the ids still present (the reference
        // rebuilds its scheduler over the remaining gates each round).
        uint64_t present = locm;
        for (int g : live) present |= ga[g];
        auto compact = [&](uint64_t m) {
            uint64_t r = 0;
            int c = 0;
            for (int b = 0; b < 64; ++b)
                if ((present >> b) & 1ULL) {
                    if ((m >> b) & 1ULL) r |= 1ULL << c;
                    ++c;
                }
            return r;
        };
        rt.resize(live.size());
        ra.resize(live.size());
        uint64_t all = compact(locm);
        for (size_t i = 0; i < live.size(); ++i) {
            rt[i] = compact(gt[live[i]]);
            ra[i] = compact(ga[live[i]]);
            all |= ra[i];
        }
        Chooser ch;
        ch.K = K;
        ch.gate = &ra;
        ch.tgt = &rt;
        ch.locals = compact(locm);
        ch.all = all;
        for (size_t i = 0; i < live.size(); ++i) {
            const uint64_t start = ch.locals & ra[i];
            if (__builtin_popcountll(start) <= K) ch.grow(start, 1);
        }
        std::vector<size_t> take;
        uint64_t blocked = 0;
        if (ch.best != 0) {
            for (size_t i = 0; i < live.size(); ++i) {
                if (ch.takeable(i, ch.best_set, blocked)) take.push_back(i);
                else blocked |= ra[i];
            }
        } else {
            for (size_t i = 0; i < live.size(); ++i) {
                if (ch.takeable(i, ch.locals, blocked)) {
                    take.push_back(i);
                    break;
                }
                blocked |= ra[i];
            }
        }
        if (take.empty()) break;
        for (size_t i : take) order[emitted++] = live[i];
        cluster_end[nclusters++] = emitted;
        std::vector<int> rest;
        rest.reserve(live.size() - take.size());
        size_t t = 0;
        for (size_t i = 0; i < live.size(); ++i) {
            if (t < take.size() && take[t] == i) {
                ++t;
                continue;
            }
            rest.push_back(live[i]);
        }
        live.swap(rest);
    }
    return nclusters;
}

}  // namespace hqs
