// Oracle (test infrastructure only) -- extern "C" entry points used by the
// tests and by the bench's CPU-baseline leg through ctypes.  Never linked
// into the product library.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "camera_math.h"
#include "residuals.h"

using namespace oracle;

namespace {

// Same field order and types as gbba_scene_t of the product ABI, so one
// ctypes structure describes both.
struct OracleScene {
  int32_t n_cameras;
  const int32_t* camera_projection;
  const double* camera_values;  // [n][16]
  int32_t n_rig_instances;
  const double* rig_instance_poses;
  int32_t n_rig_cameras;
  const double* rig_camera_poses;
  const uint8_t* rig_camera_used;
  int32_t n_shots;
  const int32_t* shot_rig_instance;
  const int32_t* shot_rig_camera;
  const int32_t* shot_camera;
  int64_t n_points;
  const double* points;
  int64_t n_observations;
  const int32_t* obs_shot;
  const int32_t* obs_point;
  const double* obs_xy;
  const double* obs_std;
};

template <typename F>
void parallel_for(int64_t n, int threads, F&& f) {
  if (threads <= 1 || n < 1024) {
    for (int64_t i = 0; i < n; ++i) f(i);
    return;
  }
  std::vector<std::thread> pool;
  const int64_t chunk = (n + threads - 1) / threads;
  for (int t = 0; t < threads; ++t) {
    const int64_t b = t * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    pool.emplace_back([b, e, &f] {
      for (int64_t i = b; i < e; ++i) f(i);
    });
  }
  for (auto& th : pool) th.join();
}

}  // namespace

extern "C" {

int oracle_num_params(int model) { return model_desc(model).n_params; }

// uv, d(uv)/d(point) 2x3 and d(uv)/d(params) 2xC with the analytic formulas.
void oracle_project(int model, const double* p, const double* params, double* uv, double* Jp,
                    double* Jc) {
  project_jac(model, p, params, uv, Jp, Jc);
}

// Same quantities by forward-mode dual numbers on the generic forward map.
void oracle_project_ad(int model, const double* p, const double* params, double* uv, double* Jp,
                       double* Jc) {
  constexpr int N = 3 + 16;
  const int C = model_desc(model).n_params;
  Dual<N> P[3], K[16];
  for (int i = 0; i < 3; ++i) P[i] = Dual<N>::var(p[i], i);
  for (int i = 0; i < C; ++i) K[i] = Dual<N>::var(params[i], 3 + i);
  Dual<N> out[2];
  project<Dual<N>>(model, P, K, out);
  for (int r = 0; r < 2; ++r) {
    uv[r] = out[r].v;
    for (int j = 0; j < 3; ++j) Jp[r * 3 + j] = out[r].d[j];
    for (int j = 0; j < C; ++j) Jc[r * C + j] = out[r].d[3 + j];
  }
}

// Residual + analytic Jacobian blocks of one observation; rig may be NULL.
void oracle_residual_jacobian(int model, const double* cam, const double* inst, const double* rig,
                              const double* X, const double* obs, double std_dev, double* r,
                              double* Jcam, double* Jinst, double* Jrig, double* Jpt) {
  residual_jac(model, cam, inst, rig, X, obs, std_dev, r, Jcam, Jinst, Jrig, Jpt);
}

// Residual + Jacobian blocks by dual numbers over [cam | inst | rig | point].
void oracle_residual_ad(int model, const double* cam, const double* inst, const double* rig,
                        const double* X, const double* obs, double std_dev, double* r,
                        double* Jcam, double* Jinst, double* Jrig, double* Jpt) {
  constexpr int N = 16 + 6 + 6 + 3;
  const int C = model_desc(model).n_params;
  const int NR = residual_size(model);
  Dual<N> K[16], I[6], G[6], P[3], out[3];
  for (int i = 0; i < C; ++i) K[i] = Dual<N>::var(cam[i], i);
  for (int i = 0; i < 6; ++i) I[i] = Dual<N>::var(inst[i], 16 + i);
  for (int i = 0; i < 6; ++i) G[i] = Dual<N>::var(rig ? rig[i] : 0.0, 22 + i);
  for (int i = 0; i < 3; ++i) P[i] = Dual<N>::var(X[i], 28 + i);
  residual_generic<Dual<N>>(model, K, I, rig ? G : nullptr, P, obs, std_dev, out);
  for (int a = 0; a < NR; ++a) {
    r[a] = out[a].v;
    for (int j = 0; j < C; ++j) Jcam[a * C + j] = model == SPHERICAL ? 0.0 : out[a].d[j];
    for (int j = 0; j < 6; ++j) Jinst[a * 6 + j] = out[a].d[16 + j];
    for (int j = 0; j < 6; ++j) Jrig[a * 6 + j] = rig ? out[a].d[22 + j] : 0.0;
    for (int j = 0; j < 3; ++j) Jpt[a * 3 + j] = out[a].d[28 + j];
  }
}

// Every observation of a scene, output blocks as gbba_evaluate_projections
// lays them out (nr rows, cmax camera columns).  Returns 0 on success.
int oracle_evaluate_scene(const OracleScene* s, int nr, int cmax, int threads, double* res,
                          double* jc, double* ji, double* jr, double* jp) {
  parallel_for(s->n_observations, threads, [&](int64_t i) {
    const int sh = s->obs_shot[i];
    const int cam = s->shot_camera[sh];
    const int model = s->camera_projection[cam];
    const int C = model_desc(model).n_params;
    const double* inst = s->rig_instance_poses + 6 * s->shot_rig_instance[sh];
    const int rc = s->shot_rig_camera[sh];
    const double* rig = (rc >= 0 && s->rig_camera_used && s->rig_camera_used[rc])
                            ? s->rig_camera_poses + 6 * rc
                            : nullptr;
    double r[3] = {0, 0, 0}, Jc[3 * 16] = {0}, Ji[18] = {0}, Jr[18] = {0}, Jp[9] = {0};
    residual_jac(model, s->camera_values + 16 * cam, inst, rig, s->points + 3 * s->obs_point[i],
                 s->obs_xy + 2 * i, s->obs_std[i], r, Jc, Ji, Jr, Jp);
    const int NR = residual_size(model);
    for (int a = 0; a < nr; ++a) {
      const bool row = a < NR;
      res[i * nr + a] = row ? r[a] : 0.0;
      if (jc)
        for (int j = 0; j < cmax; ++j) jc[(i * nr + a) * cmax + j] = (row && j < C) ? Jc[a * C + j] : 0.0;
      if (ji)
        for (int j = 0; j < 6; ++j) ji[(i * nr + a) * 6 + j] = row ? Ji[a * 6 + j] : 0.0;
      if (jr)
        for (int j = 0; j < 6; ++j) jr[(i * nr + a) * 6 + j] = row ? Jr[a * 6 + j] : 0.0;
      if (jp)
        for (int j = 0; j < 3; ++j) jp[(i * nr + a) * 3 + j] = row ? Jp[a * 3 + j] : 0.0;
    }
  });
  return 0;
}

// Robust loss rho, rho', rho'' (Ceres LossFunction definitions).
void oracle_loss(int loss, double threshold, double s, double* rho) { loss_eval(loss, threshold, s, rho); }

}  // extern "C"

extern "C" {

// PoseFunctor forward + 3x9 Jacobian [dX | d(rx,ry,rz) | d(tx,ty,tz)], analytic.
void oracle_pose_jacobian(const double* X, const double* rt, double* out, double* J) {
  pose_jac(X, rt, out, J);
}

// The same Jacobian by dual numbers on the generic forward map.
void oracle_pose_ad(const double* X, const double* rt, double* out, double* J) {
  Dual<9> P[3], T[6], o[3];
  for (int i = 0; i < 3; ++i) P[i] = Dual<9>::var(X[i], i);
  for (int i = 0; i < 6; ++i) T[i] = Dual<9>::var(rt[i], 3 + i);
  pose_forward_t<Dual<9>>(P, T, o);
  for (int i = 0; i < 3; ++i) {
    out[i] = o[i].v;
    for (int j = 0; j < 9; ++j) J[i * 9 + j] = o[i].d[j];
  }
}

}  // extern "C"
