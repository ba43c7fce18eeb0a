// Test build only (oracle/Makefile, target `adapter`): found before the reference's header of
// the same name, so that the reference's own estimator switch -- CModelAdapt::InitializeEstimator
// with the --CUDA option (lib_bmssr/trainer/OL_ModelAdapt.cpp:248-267), compiled unmodified with
// _CUDA defined -- constructs the GB300 estimator where it would construct the CUDA one. This
// stands in for the one-line `else if (_GB300acc) _estimator = new GMMStatsEstimator_GB300<...>`
// that a maintainer adds to that switch.
#ifndef _OL_STATS_EST_CUDA_
#define _OL_STATS_EST_CUDA_

#include "gb300_adapter.hpp"

template <typename TS>
class GMMStatsEstimator_CUDA : public GMMStatsEstimator_GB300<TS> {
 public:
  explicit GMMStatsEstimator_CUDA(int GPU_id = -1) : GMMStatsEstimator_GB300<TS>(GPU_id) {}
};

#endif
