// Coarse space of the two-level PCG preconditioner on the reduced camera
// system.
//
// Block-Jacobi PCG converges slowly on large aerial and street blocks: the
// slow modes are smooth motions of whole groups of cameras (a translation,
// rotation or scale of a neighbourhood), which only the GPS priors hold and
// which a 6 x 6 block per instance cannot see.  The coarse space spans those
// motions explicitly: the rig instances are split into spatial clusters
// (recursive median splits of the camera centres along the widest axis,
// at most `leaf` instances per cluster), and every cluster contributes the
// seven similarity modes of its instances about the cluster centroid g:
//   translation e_k      d centre = e_k
//   rotation e_k         d rotation = J_l^-1(r) e_k, d centre = e_k x (c - g)
//   scale                d centre = c - g
// in the camera-to-world [angle-axis r | centre c] parameters of an instance.
// The preconditioner is then
//   M^-1 = B^-1 + Z E^-1 Z^T,   E = Z^T A Z,
// B the block-Jacobi blocks and A the damped reduced camera system: SPD for
// any Z, so PCG stays valid whatever the quality of the modes.
//
// E is measured with the solver's own implicit Schur product on probe
// vectors.  Two clusters are coupled when a point is observed from both, or
// a host term (relative motion, ...) ties instances of both.  The clusters
// are coloured so that the closed neighbourhood of every cluster holds each
// colour at most once (a distance-2 colouring); then for colour k and mode
// j, A applied to the sum of mode j over all clusters of colour k gives, on
// the rows of cluster c, exactly column (partner(c, k), j) of A Z, where
// partner(c, k) is the one cluster of colour k next to c (or c itself).
// E costs 7 x (number of colours) products per linearization.
#pragma once

#include <array>
#include <cstdint>
#include <utility>
#include <vector>

#include "problem.h"

namespace gbba {

struct CoarseSpace {
  int leaf = 0;
  int n_clusters = 0, n_colours = 0;
  std::vector<int> cluster;   // per rig instance: its cluster, -1 without a free coordinate
  std::vector<int> colour;    // per cluster
  std::vector<int> partner;   // [cluster][colour]: the coupled cluster of that colour (itself included), -1
  std::vector<double> basis;  // [instance][6][7] modes; rows of locked coordinates are zero
  std::vector<std::vector<int>> neighbours;  // per cluster, sorted, itself excluded
  std::vector<int> member_start, members;    // the instances of each cluster (CSR, ascending)
  int dim() const { return 7 * n_clusters; }
};

// Largest coarse dimension the dense factorization takes; larger problems
// get larger clusters.
constexpr int kMaxCoarseDim = 4096;

// Builds the coarse space of problem P at the instances' current values.
// free_mask: per instance, six flags of its optimised coordinates (after the
// solver's own locking).  point_major: the observation indices grouped by
// point (entries < 0 are skipped), as the solver's point-major slots hold
// them.  Returns n_clusters = 0 when fewer than two clusters would form.
CoarseSpace build_coarse_space(const Problem& P, const std::vector<uint8_t>& free_mask, int leaf,
                               const std::vector<int64_t>& point_major);

// The observation indices of P grouped by point (a stable counting sort).
std::vector<int64_t> point_major_order(const Problem& P);

}  // namespace gbba
