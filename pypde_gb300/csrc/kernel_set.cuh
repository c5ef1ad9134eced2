// kernel_set.cuh -- turns a (system, order) pair into its KernelSet and a
// SystemDesc; included by the per-system instantiation units.
#pragma once

#include "batch.cuh"
#include "runtime.h"
#include "systems.cuh"

namespace pypde {

template <class Sys, int N> KernelSet make_kernel_set() {
  using Cfg = PredCfg<Sys, N>;
  KernelSet k;
  k.cfl.aot = (const void *)&k_cfl<Sys, N>;
  k.predictor.aot = (const void *)&k_predictor<Sys, N>;
  k.faces.aot = (const void *)&k_faces<Sys, N, 0>;
  k.faces_flux[0].aot = (const void *)&k_faces<Sys, N, 0>;
  k.faces_flux[1].aot = (const void *)&k_faces<Sys, N, 1>;
  k.faces_flux[2].aot = (const void *)&k_faces<Sys, N, 2>;
  k.centers.aot = (const void *)&k_centers<Sys, N>;
  k.gather.aot = (const void *)&k_gather<Sys, N>;
  k.newton.aot = (const void *)&k_newton<Sys, N>;
  k.kb_cfl.aot = (const void *)&kb_cfl<Sys, N>;
  k.kb_predictor.aot = (const void *)&kb_predictor<Sys, N>;
  k.kb_newton.aot = (const void *)&kb_newton<Sys, N>;
  k.kb_faces[0].aot = (const void *)&kb_faces<Sys, N, 0>;
  k.kb_faces[1].aot = (const void *)&kb_faces<Sys, N, 1>;
  k.kb_faces[2].aot = (const void *)&kb_faces<Sys, N, 2>;
  k.kb_centers.aot = (const void *)&kb_centers<Sys, N>;
  k.kb_gather.aot = (const void *)&kb_gather<Sys, N>;
  k.newton_threads = NewtonCfg<Sys, N>::THREADS;
  k.newton_cpb = NewtonCfg<Sys, N>::CPB;
  k.newton_smem = NewtonCfg<Sys, N>::SMEM_BYTES;
  if constexpr (MlpShape<Sys, N>::OK && Sys::HAS_S) {
    k.guess.aot = (const void *)&k_mlp_guess<Sys, N>;
    k.kb_guess.aot = (const void *)&kb_mlp_guess<Sys, N>;
    k.guess_smem = MlpShape<Sys, N>::SMEM;
    k.guess_k1 = MlpShape<Sys, N>::K1;
    k.guess_no = MlpShape<Sys, N>::NO;
    k.guess_feat = MlpShape<Sys, N>::FEAT;
  }
  if constexpr (FaceSplit<Sys>::OK) {
    k.faces_pre.aot = (const void *)&k_faces_pre<Sys, N>;
    k.faces_eig.aot = (const void *)&k_faces_eig<Sys, N>;
    k.face_rec = FaceSplit<Sys>::REC;
    k.kb_faces_pre.aot = (const void *)&kb_faces_pre<Sys, N>;
    k.kb_faces_eig.aot = (const void *)&kb_faces_eig<Sys, N>;
  }
  k.pred_threads = Cfg::THREADS;
  k.pred_cpb = Cfg::CPB;
  k.pred_smem = (size_t)Cfg::SMEM_DOUBLES * sizeof(double);
  return k;
}

template <class Sys, int... Ns> SystemDesc describe(const char *name) {
  SystemDesc d;
  d.name = name;
  d.ndim = Sys::NDIM;
  d.V = Sys::V;
  d.has_F = Sys::HAS_F;
  d.has_B = Sys::HAS_B;
  d.has_S = Sys::HAS_S;
  d.second_order = Sys::SECOND_ORDER;
  int ns[] = {Ns...};
  KernelSet ks[] = {make_kernel_set<Sys, Ns>()...};
  for (unsigned i = 0; i < sizeof(ns) / sizeof(ns[0]); i++) {
    d.sets[ns[i]] = ks[i];
    d.have[ns[i]] = true;
  }
  return d;
}

} // namespace pypde
