// placement.cpp -- device placement for the three splits of corr_cuda.h.
//
// The splits and what each device must report through corr_device_plan_get /
// corr_device_stations / corr_device_baselines follow the reference
// (corr-cuda/src/corr_cuda.cpp:180-470, checked by corr-cuda/tests/multi_device.c):
// time slice and baseline range give every device every station; pair covering
// gives each device a proper subset and each baseline to exactly one device
// that holds both of its stations.
//
// Pair covering is built here from groups rather than by search. The stations
// are cut into m contiguous groups of near-equal size, m the largest number
// with m(m-1)/2 <= n_devices. Device d holds the union of the d-th unordered
// pair of groups {a, b} (a < b, in lexicographic order; devices beyond the
// m(m-1)/2 pairs take the pairs again from the first). Every two groups meet on
// some device, so every baseline is computable somewhere; each is given to the
// device, among those able to compute it, that owns the fewest so far (baselines
// across two groups first, since fewer devices can take them). Each
// device holds two groups, so resident sets differ by at most one station (the
// groups differ by at most one), and no device holds every station once there
// are three or more devices. The host-link replication factor is 2*n_devices/m
// (2.67 at 4 devices, 3 at 6, 2 at 3); with two devices both must hold every
// station, since two proper subsets cannot meet every pair.

#include "placement.h"

#include <algorithm>
#include <cstring>

#include "engine.h"

namespace corrgb {
namespace {

int pair_index(int j, int k, int n) {   // j <= k, row-major over j <= k
    return j * n - j * (j - 1) / 2 + (k - j);
}

void finish(DevicePlacement *pl) {
    pl->contiguous = true;
    for (size_t i = 1; i < pl->baselines.size(); ++i)
        if (pl->baselines[i] != pl->baselines[i - 1] + 1) pl->contiguous = false;
}

DevicePlacement every_station(int ordinal, int n) {
    DevicePlacement pl;
    pl.ordinal = ordinal;
    for (int s = 0; s < n; ++s) pl.stations.push_back(s);
    return pl;
}

void plan_time_slice(int n, const std::vector<int> &ordinals, std::vector<DevicePlacement> *out) {
    const int nb = n * (n + 1) / 2;
    for (int ord : ordinals) {
        DevicePlacement pl = every_station(ord, n);
        for (int b = 0; b < nb; ++b) {
            pl.baselines.push_back(b);
            pl.local.push_back(b);
        }
        finish(&pl);
        out->push_back(std::move(pl));
    }
}

void plan_range(int n, const std::vector<int> &ordinals, std::vector<DevicePlacement> *out) {
    const int nb = n * (n + 1) / 2;
    const int nd = static_cast<int>(ordinals.size());
    int first = 0;
    for (int d = 0; d < nd; ++d) {
        const int count = nb / nd + (d < nb % nd ? 1 : 0);
        DevicePlacement pl = every_station(ordinals[static_cast<size_t>(d)], n);
        for (int b = first; b < first + count; ++b) {
            pl.baselines.push_back(b);
            pl.local.push_back(b);   // every station held: local numbering = global
        }
        first += count;
        finish(&pl);
        out->push_back(std::move(pl));
    }
}

void plan_pair_covering(int n, const std::vector<int> &ordinals,
                        std::vector<DevicePlacement> *out) {
    const int nd = static_cast<int>(ordinals.size());
    if (nd == 1) {
        plan_time_slice(n, ordinals, out);
        return;
    }
    int m = 2;
    while ((m + 1) * m / 2 <= nd && m + 1 <= n) ++m;
    auto group_of = [&](int s) { return static_cast<int>(static_cast<long long>(s) * m / n); };
    std::vector<std::pair<int, int>> blocks;
    for (int a = 0; a < m; ++a)
        for (int b = a + 1; b < m; ++b) blocks.emplace_back(a, b);
    std::vector<std::pair<int, int>> held(static_cast<size_t>(nd));
    for (int d = 0; d < nd; ++d) {
        held[static_cast<size_t>(d)] = blocks[static_cast<size_t>(d) % blocks.size()];
        DevicePlacement pl;
        pl.ordinal = ordinals[static_cast<size_t>(d)];
        for (int s = 0; s < n; ++s) {
            const int g = group_of(s);
            if (g == held[static_cast<size_t>(d)].first || g == held[static_cast<size_t>(d)].second)
                pl.stations.push_back(s);
        }
        out->push_back(std::move(pl));
    }
    // local index of station s on device d (stations ascending)
    auto local_station = [&](int d, int s) {
        const auto &st = (*out)[static_cast<size_t>(d)].stations;
        return static_cast<int>(std::lower_bound(st.begin(), st.end(), s) - st.begin());
    };
    // Baselines across two groups can go only to the devices holding that pair
    // of groups; those within one group (autocorrelations included) to any
    // device holding the group. The constrained ones are placed first, then the
    // rest fill the least-loaded devices.
    for (int pass = 0; pass < 2; ++pass)
        for (int j = 0; j < n; ++j)
            for (int k = j; k < n; ++k) {
                const int gj = group_of(j), gk = group_of(k);
                if ((gj != gk) != (pass == 0)) continue;
                int best = -1;
                size_t fewest = 0;
                for (int d = 0; d < nd; ++d) {
                    const auto h = held[static_cast<size_t>(d)];
                    const bool has_j = gj == h.first || gj == h.second;
                    const bool has_k = gk == h.first || gk == h.second;
                    if (!has_j || !has_k) continue;
                    const size_t owned = (*out)[static_cast<size_t>(d)].baselines.size();
                    if (best < 0 || owned < fewest) {
                        best = d;
                        fewest = owned;
                    }
                }
                DevicePlacement &pl = (*out)[static_cast<size_t>(best)];
                const int nl = static_cast<int>(pl.stations.size());
                pl.baselines.push_back(pair_index(j, k, n));
                pl.local.push_back(pair_index(local_station(best, j), local_station(best, k), nl));
            }
    // report each device's baselines in ascending global order
    for (auto &pl : *out) {
        std::vector<std::pair<int32_t, int32_t>> bl;
        for (size_t i = 0; i < pl.baselines.size(); ++i) bl.emplace_back(pl.baselines[i], pl.local[i]);
        std::sort(bl.begin(), bl.end());
        for (size_t i = 0; i < bl.size(); ++i) {
            pl.baselines[i] = bl[i].first;
            pl.local[i] = bl[i].second;
        }
    }
    for (auto &pl : *out) finish(&pl);
}

} // namespace

corr_status plan_devices(int n_station, int split_mode, const std::vector<int> &ordinals,
                         std::vector<DevicePlacement> *out) {
    out->clear();
    if (ordinals.empty()) return fail(CORR_ERR_ARG, "no device to place the run on");
    if (n_station < 1) return fail(CORR_ERR_ARG, "n_station must be >= 1");
    if (split_mode == CORR_SPLIT_TIME_SLICE)
        plan_time_slice(n_station, ordinals, out);
    else if (split_mode == CORR_SPLIT_BASELINE_RANGE)
        plan_range(n_station, ordinals, out);
    else if (split_mode == CORR_SPLIT_PAIR_COVERING)
        plan_pair_covering(n_station, ordinals, out);
    else
        return failf(CORR_ERR_ARG, "split_mode=%d is not a known split", split_mode);
    for (size_t d = 0; d < out->size(); ++d)
        if ((*out)[d].baselines.empty()) {
            out->clear();
            return failf(CORR_ERR_ARG,
                         "the split gives device index %zu no baselines (%d stations over %zu "
                         "devices); use fewer devices",
                         d, n_station, ordinals.size());
        }
    return CORR_OK;
}

corr_status check_device_baselines(const std::vector<DevicePlacement> &plan) {
    for (size_t d = 0; d < plan.size(); ++d)
        if (plan[d].baselines.size() > static_cast<size_t>(kMaxBaselinesPerDevice))
            return failf(CORR_ERR_ARG,
                         "device index %zu would own %zu baselines; at most %d per device "
                         "(n_station <= 44 on one device; split the baselines over more "
                         "devices)",
                         d, plan[d].baselines.size(), kMaxBaselinesPerDevice);
    return CORR_OK;
}

bool placement_is_identity(const DevicePlacement &pl, int n_station) {
    const size_t nb = static_cast<size_t>(n_station) * (n_station + 1) / 2;
    if (pl.stations.size() != static_cast<size_t>(n_station) || pl.baselines.size() != nb)
        return false;
    for (size_t i = 0; i < nb; ++i)
        if (pl.baselines[i] != static_cast<int32_t>(i) || pl.local[i] != static_cast<int32_t>(i))
            return false;
    return true;
}

void fill_device_plan(const DevicePlacement &pl, corr_device_plan *out) {
    out->device_id = pl.ordinal;
    out->n_station_resident = static_cast<int32_t>(pl.stations.size());
    out->first_baseline = pl.baselines.empty() ? 0 : pl.baselines.front();
    out->n_baseline = static_cast<int32_t>(pl.baselines.size());
    out->contiguous = pl.contiguous ? 1 : 0;
}

} // namespace corrgb

using namespace corrgb;

extern "C" corr_status corrx_plan_query(const corr_config *cfg, int32_t device_index,
                                        corr_device_plan *out, int32_t *out_stations,
                                        int32_t stations_len, int32_t *out_baselines,
                                        int32_t baselines_len, int32_t *out_local,
                                        int32_t local_len) {
    if (cfg == nullptr || out == nullptr) return fail(CORR_ERR_ARG, "cfg and out must be non-NULL");
    if (cfg->abi_version != CORR_ABI_VERSION || cfg->struct_size != sizeof(corr_config))
        return fail(CORR_ERR_ABI, "abi_version / struct_size mismatch");
    if (cfg->n_devices < 0 || cfg->n_devices > static_cast<int32_t>(CORR_MAX_DEVICES))
        return failf(CORR_ERR_ARG, "n_devices=%d outside [0, %u]", cfg->n_devices,
                     CORR_MAX_DEVICES);
    if (cfg->n_station < 1 || cfg->n_station > kMaxStations)
        return failf(CORR_ERR_ARG, "n_station must be in [1, %d]", kMaxStations);
    std::vector<int> ordinals;
    if (cfg->n_devices > 0)
        ordinals.assign(cfg->devices, cfg->devices + cfg->n_devices);
    else
        ordinals.push_back(cfg->device_id);
    std::vector<DevicePlacement> plan;
    corr_status st = plan_devices(cfg->n_station, cfg->split_mode, ordinals, &plan);
    if (st != CORR_OK) return st;
    if ((st = check_device_baselines(plan)) != CORR_OK) return st;
    if (device_index < 0 || device_index >= static_cast<int32_t>(plan.size()))
        return failf(CORR_ERR_ARG, "device_index %d out of range [0,%zu)", device_index,
                     plan.size());
    const DevicePlacement &pl = plan[static_cast<size_t>(device_index)];
    fill_device_plan(pl, out);
    auto put = [](const std::vector<int32_t> &v, int32_t *dst, int32_t len) -> bool {
        if (dst == nullptr) return true;
        if (len < static_cast<int32_t>(v.size())) return false;
        std::copy(v.begin(), v.end(), dst);
        return true;
    };
    if (!put(pl.stations, out_stations, stations_len) ||
        !put(pl.baselines, out_baselines, baselines_len) || !put(pl.local, out_local, local_len))
        return fail(CORR_ERR_ARG, "an output array is shorter than the plan");
    return CORR_OK;
}
