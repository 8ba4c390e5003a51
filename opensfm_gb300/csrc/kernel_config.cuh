// Kernel configurations of the solver's record passes: a single camera
// model (compile-time model, residual rows and intrinsics width), or the
// dynamic configuration (runtime model per camera, 16 intrinsics columns,
// optional rig-camera columns, 2 or 3 residual rows).
#pragma once

#include "camera_models.cuh"

namespace gbba {

constexpr int kDyn = -1;

struct KernelConfig {
  int model;  // single model or kDyn
  int nr;
  int cmax;
  bool rig;
};

// Calls f.template run<M, NR, CMAX, RIG>() for a kernel configuration.
template <typename F>
void dispatch_config(const KernelConfig& k, F& f) {
  if (k.model != kDyn) {
    switch (k.model) {
      case kPerspective: f.template run<kPerspective, 2, 3, false>(); return;
      case kBrown: f.template run<kBrown, 2, 9, false>(); return;
      case kFisheye: f.template run<kFisheye, 2, 3, false>(); return;
      case kFisheyeOpencv: f.template run<kFisheyeOpencv, 2, 8, false>(); return;
      case kFisheye62: f.template run<kFisheye62, 2, 12, false>(); return;
      case kFisheye624: f.template run<kFisheye624, 2, 16, false>(); return;
      case kDual: f.template run<kDual, 2, 4, false>(); return;
      case kRadial: f.template run<kRadial, 2, 6, false>(); return;
      case kSimpleRadial: f.template run<kSimpleRadial, 2, 5, false>(); return;
    }
  }
  if (k.nr == 2) {
    if (k.rig) f.template run<kDyn, 2, 16, true>();
    else f.template run<kDyn, 2, 16, false>();
  } else {
    if (k.rig) f.template run<kDyn, 3, 16, true>();
    else f.template run<kDyn, 3, 16, false>();
  }
}

}  // namespace gbba
