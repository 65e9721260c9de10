// placement.h -- which stations each device of a context holds and which
// baselines it owns, for the three splits of corr_cuda.h (CORR_SPLIT_*).
//
// Host-only: no CUDA call, so the planner can be queried and tested on a
// machine without a GPU (corrx_plan_query).

#ifndef CORR_GB300_PLACEMENT_H
#define CORR_GB300_PLACEMENT_H

#include <cstdint>
#include <vector>

#include "corr_cuda.h"

namespace corrgb {

/// One device's share of a run.
struct DevicePlacement {
    int ordinal = 0;                  // configured device (corr_config.devices[i])
    std::vector<int32_t> stations;    // global station indices, ascending; local i = stations[i]
    std::vector<int32_t> baselines;   // global baselines this device reports, ascending
    std::vector<int32_t> local;       // for each of them, its index among the device's
                                      // local baselines (j <= k over `stations`, row-major)
    bool contiguous = true;           // baselines form one ascending run
};

/// Placement of n_station stations over the devices `ordinals` for a split:
///   CORR_SPLIT_TIME_SLICE: every device holds every station and reports every
///     baseline, as a partial row over the slots routed to it (seq % n_devices);
///   CORR_SPLIT_BASELINE_RANGE: every device holds every station and reports a
///     contiguous range of the baselines, B/n_devices each, the remainder going
///     one each to the first devices;
///   CORR_SPLIT_PAIR_COVERING: each device holds a subset of the stations and
///     reports baselines among them, every baseline exactly once (below).
/// CORR_ERR_ARG when a device would report no baseline.
corr_status plan_devices(int n_station, int split_mode, const std::vector<int> &ordinals,
                         std::vector<DevicePlacement> *out);

/// The reference's per-device limit (corr-cuda/src/kernels.cu:474-483): every
/// device owns at most kMaxBaselinesPerDevice baselines, so a run of more than
/// 44 stations needs its baselines split over several devices.
corr_status check_device_baselines(const std::vector<DevicePlacement> &plan);

/// Whether the placement is one device's whole row in order (no gather needed).
bool placement_is_identity(const DevicePlacement &pl, int n_station);

void fill_device_plan(const DevicePlacement &pl, corr_device_plan *out);

} // namespace corrgb

#endif // CORR_GB300_PLACEMENT_H
