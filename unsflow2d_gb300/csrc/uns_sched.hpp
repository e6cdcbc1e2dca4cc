// uns_sched.hpp -- host-side warp schedule of the LU-SGS sweeps.
//
// The forward sweep of lusgs2 (CCFVM/lusgs.F90:245-280, NCFVM/lusgs.f90:48-86)
// updates entity i from its already-updated neighbours j < i; the backward
// sweep (CCFVM/lusgs.F90:283-318, NCFVM/lusgs.f90:88-124) from j > i and from
// i's own forward value.  Each (entity, pass) is one item of a DAG whose
// longest path is long (thousands of items on an O-mesh), so the sweep is
// latency-bound: what matters is how fast one item can follow another.
//
// An item that follows a predecessor computed by the same warp takes its
// values from registers; one that follows another warp's item must see that
// item's published record in L2.  list_schedule assigns the items to warps by
// greedy list scheduling on that cost model (an item costs kCompute; a
// cross-warp edge adds kSync): each item, in topological order, goes to the
// warp of its last-finishing predecessor when that warp has nothing newer
// queued, else to the warp that frees up first, whichever starts it earlier.
//
// Each warp's list is in increasing simulated start time and every
// dependency of an item has a strictly earlier simulated start, so with all
// warps resident (cooperative launch) the lowest-start unfinished item can
// always proceed: the sweep cannot deadlock.
#pragma once
#include <algorithm>
#include <cstdlib>
#include <functional>
#include <queue>
#include <utility>
#include <vector>

namespace uns {

struct WarpSchedule {
    std::vector<int> off;    // nwarps + 1 offsets into items
    std::vector<int> items;  // (entity << 1) | pass, pass 0 = forward, 1 = backward
    double makespan = 0.0;   // simulated length in units of one item's compute
    int nlev_fwd = 0, nlev_bwd = 0;
};

// nbr_off / nbr: CSR neighbour lists of the n entities (any order, entries
// outside [0, n) ignored).  nwarps: warps of the cooperative launch.  kSync:
// the extra delay of a cross-warp dependency, in units of one item's compute.
inline WarpSchedule list_schedule(int n, const int* nbr_off, const int* nbr, int nwarps, double kSync = 0.25) {
    constexpr double kCompute = 1.0;
    // Topological orders: forward by dependency level (then index), backward
    // by backward level (then descending index).
    std::vector<int> lev(n, 0), levb(n, 0);
    int nlev = 0, nlevb = 0;
    for (int i = 0; i < n; ++i) {
        int l = 0;
        for (int k = nbr_off[i]; k < nbr_off[i + 1]; ++k) {
            int j = nbr[k];
            if (j >= 0 && j < i) l = std::max(l, lev[j] + 1);
        }
        lev[i] = l;
        nlev = std::max(nlev, l + 1);
    }
    for (int i = n - 1; i >= 0; --i) {
        int l = 0;
        for (int k = nbr_off[i]; k < nbr_off[i + 1]; ++k) {
            int j = nbr[k];
            if (j > i && j < n) l = std::max(l, levb[j] + 1);
        }
        levb[i] = l;
        nlevb = std::max(nlevb, l + 1);
    }
    std::vector<int> fwd(n), bwd(n);
    {
        std::vector<int> cnt(nlev + 1, 0);
        for (int i = 0; i < n; ++i) ++cnt[lev[i] + 1];
        for (int l = 0; l < nlev; ++l) cnt[l + 1] += cnt[l];
        for (int i = 0; i < n; ++i) fwd[cnt[lev[i]]++] = i;
        std::vector<int> cb(nlevb + 1, 0);
        for (int i = 0; i < n; ++i) ++cb[levb[i] + 1];
        for (int l = 0; l < nlevb; ++l) cb[l + 1] += cb[l];
        for (int i = n - 1; i >= 0; --i) bwd[cb[levb[i]]++] = i;
    }

    std::vector<double> fin(2 * (size_t)n, 0.0);  // item code -> simulated finish
    std::vector<int> wof(2 * (size_t)n, -1);      // item code -> warp
    std::vector<double> wfree(nwarps, 0.0);
    std::vector<int> wlast(nwarps, -1);
    std::vector<std::vector<int>> lists(nwarps);
    using E = std::pair<double, int>;
    std::priority_queue<E, std::vector<E>, std::greater<E>> heap;
    for (int w = 0; w < nwarps; ++w) heap.push({0.0, w});

    std::vector<int> preds;
    auto place = [&](int code) {
        // ready time of the item on warp w
        auto start_on = [&](int w) {
            double s = wfree[w];
            for (int p : preds) s = std::max(s, fin[p] + (wof[p] == w ? 0.0 : kSync));
            return s;
        };
        // candidate warps: those whose newest item is a predecessor (the
        // chain continues there); ties go to the predecessor nearest in
        // index, so chains follow the mesh numbering where they can
        const int self = code >> 1;
        int wa = -1, da = 0;
        double sa = 0.0;
        for (int p : preds) {
            int w = wof[p];
            if (wlast[w] != p) continue;
            double s = start_on(w);
            int dist = std::abs((p >> 1) - self);
            if (wa < 0 || s < sa || (s == sa && dist < da)) { wa = w; sa = s; da = dist; }
        }
        while (heap.top().first != wfree[heap.top().second]) heap.pop();  // drop stale entries
        int wb = heap.top().second;
        double sb = start_on(wb);
        int w = wb;
        double s = sb;
        if (wa >= 0 && sa <= sb) { w = wa; s = sa; }
        fin[code] = s + kCompute;
        wof[code] = w;
        wfree[w] = fin[code];
        wlast[w] = code;
        heap.push({wfree[w], w});
        lists[w].push_back(code);
    };
    for (int i : fwd) {
        preds.clear();
        for (int k = nbr_off[i]; k < nbr_off[i + 1]; ++k) {
            int j = nbr[k];
            if (j >= 0 && j < i) preds.push_back(2 * j);
        }
        place(2 * i);
    }
    for (int i : bwd) {
        preds.clear();
        preds.push_back(2 * i);  // own forward value
        for (int k = nbr_off[i]; k < nbr_off[i + 1]; ++k) {
            int j = nbr[k];
            if (j > i && j < n) preds.push_back(2 * j + 1);
        }
        place(2 * i + 1);
    }
    WarpSchedule out;
    out.makespan = fin.empty() ? 0.0 : *std::max_element(fin.begin(), fin.end());
    out.nlev_fwd = nlev;
    out.nlev_bwd = nlevb;
    out.off.assign(nwarps + 1, 0);
    for (int w = 0; w < nwarps; ++w) out.off[w + 1] = out.off[w] + (int)lists[w].size();
    out.items.reserve(2 * (size_t)n);
    for (int w = 0; w < nwarps; ++w) out.items.insert(out.items.end(), lists[w].begin(), lists[w].end());
    return out;
}

}  // namespace uns
