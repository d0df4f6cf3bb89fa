// check_immunity (immunity.py:303-350) for one agent, shared by the fused agent
// pass, infect()'s severe-efficacy lookup and the standalone drop-ins, so that
// every path forms the efficacies with the same operations.
#pragma once
#include <stdint.h>
#include "covgpu.h"
#include "covgpu_device.cuh"
#include "covgpu_ff.cuh"

namespace covgpu {

// The immunity of agent i against variant v: the larger of the natural immunity
// (immunity[v, recovered_variant] once t >= date_recovered; was_inf and rv are
// those two inputs) and the vaccine's (vx_imm[vaccine_source, v] when
// vaccinated, flags f), with its natural logarithm from the host's tables.
__device__ __forceinline__ float imm_of(const covgpu_state& st, const covgpu_sim_params& sp, int64_t i, int v,
                                        uint32_t f, bool was_inf, uint32_t rv, ff& ln_imm) {
  const int nv = sp.n_variants;
  float imm = 0.0f;
  ln_imm = ff{0.0f, 0.0f};
  if (was_inf && rv < (uint32_t)nv) {
    const int q = v * COVGPU_MAX_VARIANTS + (int)rv;
    imm = sp.immunity[q];
    ln_imm = ff{sp.ln_immunity[q][0], sp.ln_immunity[q][1]};
  }
  if ((f & B_VACC) && sp.vx_imm && sp.vx_ln_imm) {
    const int src = st.vaccine_source[i];
    if (src >= 0 && src < sp.n_vaccines && sp.vx_imm[src * nv + v] > imm) {
      imm = sp.vx_imm[src * nv + v];
      ln_imm = ff{sp.vx_ln_imm[2 * (src * nv + v)], sp.vx_ln_imm[2 * (src * nv + v) + 1]};
    }
  }
  return imm;
}

// symp_imm of agent i against variant v as check_immunity (immunity.py:303-350)
// leaves it: 0 for an agent that never had NAbs (peak_nab 0), whose efficacies
// the agent pass does not rewrite each day
__device__ __forceinline__ float symp_imm_of(const covgpu_state& st, int64_t i, int v) {
  return st.peak_nab[i] == 0.0f ? 0.0f : st.symp_imm[(int64_t)v * st.n + i];
}

// calc_VE (immunity.py:216-247) of axis k (0 sus, 1 symp, 2 sev) for ln(nab * imm)
__device__ __forceinline__ float ve_axis(const covgpu_sim_params& sp, int k, ff ln_eff, const float (*etab)[2]) {
  return ve_ff(ln_eff, ff{sp.ve_alpha[k][0], sp.ve_alpha[k][1]}, ff{sp.ve_beta[k][0], sp.ve_beta[k][1]}, etab);
}

}  // namespace covgpu
