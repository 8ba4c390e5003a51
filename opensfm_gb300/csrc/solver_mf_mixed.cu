// Matrix-free record passes of the mixed-precision solver: every pass
// evaluates the observations' residual + Jacobian records again instead of
// reading stored ones (see record_source.cuh).
#include "record_passes.cuh"

namespace gbba {
namespace {

template <typename R>
struct EvaluatedLaunch {
  const RecordPassArgs<R>& a;
  template <int M, int NR, int CMAX, bool RIG>
  void run() {
    a.template launch<M, NR, CMAX, RIG>(EvaluatedRecords<R, M, NR, CMAX, RIG>{});
  }
};

}  // namespace

template <>
void launch_evaluated<float>(const KernelConfig& kc, const RecordPassArgs<float>& a) {
  EvaluatedLaunch<float> f{a};
  dispatch_config(kc, f);
}

}  // namespace gbba
