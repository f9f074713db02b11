// lif.cuh -- one exponential-Euler step of a LifRefLTC / LifRef neuron with two Expon+COBA
// conductance channels, in float32 with every operation rounded as written (no contraction),
// so that GPU and CPU results agree bit for bit.
//
//   Expon (brainpy/_src/dyn/synapses/abstract_models.py:121-134):
//     g += dg (add_current, the projection's event sum);  g <- g + (dt*exprel(dt*lin)) * ((-g)/tau),
//     lin = d(-g/tau)/dg = -(1/tau)
//   COBA (brainpy/_src/dyn/outs/outputs.py:53-54): I_k = g_k * (E_k - V)
//   LifRefLTC (brainpy/_src/dyn/neurons/lif.py:461-500, derivative :254-256):
//     I = (inp + ge*(Ee - V)) + gi*(Ei - V);  f = ((-V + V_rest) + R*I) / tau
//     lin = (-1 - R*(ge + gi)) / tau        (LifRef, lif.py:550-556: lin = -(1/tau))
//     V' = V + (dt*exprel(dt*lin)) * f      (brainpy/_src/integrators/ode/exponential.py:357-362)
//     refractory (t - t_last) <= tau_ref keeps V; spike = V' >= V_th; reset; t_last = t on spike
#pragma once

#include "../../include/bpgpu.h"
#include "bp_math.h"

namespace bp {

struct LifState {
  float V, ge, gi, t_last;
};

__device__ __forceinline__ bool lif_coba_update(const bp_lif_params& p, LifState& s, float dge, float dgi, float t,
                                                float dt) {
  float g_e = BP_FADD(s.ge, dge);
  float g_i = BP_FADD(s.gi, dgi);
  {
    const float lin = -BP_FDIV(1.0f, p.tau_e);
    const float dtphi = BP_FMUL(dt, bp_exprel(BP_FMUL(dt, lin)));
    g_e = BP_FADD(g_e, BP_FMUL(dtphi, BP_FDIV(-g_e, p.tau_e)));
  }
  {
    const float lin = -BP_FDIV(1.0f, p.tau_i);
    const float dtphi = BP_FMUL(dt, bp_exprel(BP_FMUL(dt, lin)));
    g_i = BP_FADD(g_i, BP_FMUL(dtphi, BP_FDIV(-g_i, p.tau_i)));
  }
  const float v = s.V;
  const float I = BP_FADD(BP_FADD(p.input, BP_FMUL(g_e, BP_FSUB(p.E_e, v))), BP_FMUL(g_i, BP_FSUB(p.E_i, v)));
  const float f = BP_FDIV(BP_FADD(BP_FADD(-v, p.V_rest), BP_FMUL(p.R, I)), p.tau);
  float lin;
  if (p.ltc) lin = BP_FDIV(BP_FSUB(-1.0f, BP_FMUL(p.R, BP_FADD(g_e, g_i))), p.tau);
  else lin = -BP_FDIV(1.0f, p.tau);
  const float phi = bp_exprel(BP_FMUL(dt, lin));
  float vn = BP_FADD(v, BP_FMUL(BP_FMUL(dt, phi), f));
  if (BP_FSUB(t, s.t_last) <= p.tau_ref) vn = v;
  const bool spike = vn >= p.V_th;
  if (spike) {
    vn = p.V_reset;
    s.t_last = t;
  }
  s.V = vn;
  s.ge = g_e;
  s.gi = g_i;
  return spike;
}

}  // namespace bp
