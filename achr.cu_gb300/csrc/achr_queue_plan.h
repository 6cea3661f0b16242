// Work items of one persistent work-queue launch (host code, no CUDA types):
// the chains of the models that share a chain-kernel configuration, cut into
// tiles (model, first chain, end chain).  Models run longest chain time first;
// each tile holds the work still queued behind it divided by tiles x ctas
// (guided self-scheduling), so early tiles are large (few queue operations)
// and the last ones are single chains, and the CTAs leave the queue within
// about one chain's time of each other.
#pragma once

#include <algorithm>
#include <vector>

namespace achr {

struct QueueItem {
    int model, p0, p1;
};

// models: indices into n_points / chain_time; ctas: resident CTAs of the launch.
inline std::vector<QueueItem> plan_queue(std::vector<int> models, const int *n_points, const double *chain_time,
                                         int ctas, int tiles) {
    std::vector<QueueItem> items;
    double left = 0.0;
    for (int k : models) left += (double)n_points[k] * chain_time[k];
    std::stable_sort(models.begin(), models.end(), [&](int x, int y) { return chain_time[x] > chain_time[y]; });
    const double per = (double)std::max(1, tiles) * (double)std::max(1, ctas);
    for (int k : models) {
        const double t = std::max(chain_time[k], 1e-30);
        for (int p = 0; p < n_points[k];) {
            long long tile = (long long)(left / (per * t));
            tile = std::max(1LL, std::min(tile, (long long)(n_points[k] - p)));
            items.push_back(QueueItem{k, p, p + (int)tile});
            p += (int)tile;
            left -= (double)tile * t;
        }
    }
    return items;
}

}  // namespace achr
