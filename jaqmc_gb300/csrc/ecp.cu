// Effective-core-potential energy (qmc_ecp_energy): the reference's ECPEnergy
// estimator (src/jaqmc/estimator/ecp/estimator.py:33-155) with its radial
// potentials (:158-275), nearest-core selection (:278-320) and nonlocal
// integral over rotated spherical quadrature points
// (src/jaqmc/estimator/ecp/nonlocal_integral.py:17-130).
//
//   E_ecp = sum_{i,I} V_0(r_iI)
//         + sum_i sum_{I in the max_core nearest} sum_l V_{l+1}(r_iI) (2l + 1)
//             sum_q w_q P_l(cos theta_q) psi(.., r_i^q, ..) / psi(..)
//   r_i^q = R_I + |r_i - R_I| Rot_i x_q,  cos theta_q = (Rot_i x_q) . (r_i - R_I) / |r_i - R_I|
//
// Every displaced configuration is a full forward pass (the FermiNet's spin
// means make every orbital depend on every electron), so the work is
// batch x n x max_core x n_quad forwards; they run through the model's own
// forward (qmc_forward's kernels) in chunks of at most kEcpConfigs
// configurations, each chunk a contiguous range of walkers.
#include "common.cuh"
#include "plan.cuh"
#include "profile.cuh"
#include "psiformer.cuh"

namespace qmc {

template <typename T>
static T* at(void* ws, size_t off) { return reinterpret_cast<T*>(static_cast<char*>(ws) + off); }

constexpr int kEcpConfigs = 65536;   // configurations per forward chunk
constexpr int kEcpMaxChannels = 5;   // local + s, p, d, f
constexpr int kEcpMaxCore = 8;

struct EcpShape {
  int B, n, MC, Q, L;  // L: nonlocal channels
  int Wc;              // walkers per chunk
  size_t sel, vnl, dir, rad, rot, lp0, sg0, cfg, lp1, sg1, fwd, total;
};

static EcpShape ecp_shape(const qmc_model* m, int B, int MC, int Q, int L) {
  EcpShape e{};
  const int n = m->d.n;
  e.B = B;
  e.n = n;
  e.MC = MC;
  e.Q = Q;
  e.L = L;
  const long per_w = (long)n * MC * Q;
  e.Wc = (int)std::max<long>(1, std::min<long>(B, kEcpConfigs / std::max<long>(per_w, 1)));
  const size_t G = (size_t)e.Wc * per_w;
  size_t o = 0;
  auto take = [&](size_t bytes) { size_t r = o; o += align_up(bytes, 256); return r; };
  const size_t pairs = (size_t)B * n * MC;
  e.sel = take(pairs * 4);
  e.vnl = take(pairs * (L > 0 ? L : 1) * 4);
  e.dir = take(pairs * 3 * 4);
  e.rad = take(pairs * 4);
  e.rot = take((size_t)B * n * 9 * 4);
  e.lp0 = take((size_t)B * 4);
  e.sg0 = take((size_t)B * 4);
  e.cfg = take(G * n * 3 * 4);
  e.lp1 = take(G * 4);
  e.sg1 = take(G * 4);
  const size_t fwd_w = std::max<size_t>(G, (size_t)e.Wc);
  const size_t fwd = m->kind == QMC_KIND_PSIFORMER ? psi_make_plan(m, (int)fwd_w).base.total
                                                   : make_plan(m, QMC_OP_FORWARD, (int)fwd_w).total;
  e.fwd = take(fwd);
  e.total = o;
  return e;
}

// Per (walker, electron): rotation (given or from Philox), local energy
// contribution, and the max_core nearest ECP atoms with their nonlocal radial
// values, unit directions and distances.  One block per walker, a thread per
// electron; the local sum is reduced in the block.
__global__ void k_ecp_prepare(int n, int A, int Ae, int C, int T, int MC, const float* __restrict__ x,
                              const float* __restrict__ atoms, const int* __restrict__ ecp_atoms,
                              const float* __restrict__ radial, const float* __restrict__ rot_in, uint64_t seed,
                              uint64_t counter, float* __restrict__ e_local, int* __restrict__ sel,
                              float* __restrict__ vnl, float* __restrict__ dir, float* __restrict__ rad,
                              float* __restrict__ rot) {
  extern __shared__ float red[];
  const int w = blockIdx.x;
  float loc = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const float* xi = x + ((size_t)w * n + i) * 3;
    float* R = rot + ((size_t)w * n + i) * 9;
    if (rot_in) {
      for (int k = 0; k < 9; ++k) R[k] = rot_in[((size_t)w * n + i) * 9 + k];
    } else {
      // phi = 2 pi u1, cos theta = 1 - 2 u2 (quadrature.py, sample_rotation_matrices)
      const U4 r = philox4x32_10(U4{0x80000000u | (uint32_t)i, (uint32_t)w, (uint32_t)counter,
                                    (uint32_t)(counter >> 32)},
                                 (uint32_t)seed, (uint32_t)(seed >> 32));
      const float phi = 6.283185307179586f * u01(r.x);
      const float ct = 1.f - 2.f * u01(r.y);
      const float st = sqrtf(fmaxf(0.f, 1.f - ct * ct));
      float sp, cp;
      sincosf(phi, &sp, &cp);
      R[0] = sp * sp + ct * cp * cp;
      R[1] = sp * cp * (ct - 1.f);
      R[2] = st * cp;
      R[3] = sp * cp * (ct - 1.f);
      R[4] = cp * cp + ct * sp * sp;
      R[5] = st * sp;
      R[6] = -st * cp;
      R[7] = -st * sp;
      R[8] = ct;
    }
    // nearest ECP atoms by insertion (ties keep the lower index, as a stable sort)
    int best[kEcpMaxCore];
    float bd[kEcpMaxCore];
    for (int c = 0; c < MC; ++c) {
      best[c] = -1;
      bd[c] = INFINITY;
    }
    for (int a = 0; a < Ae; ++a) {
      const int ai = ecp_atoms[a];
      if (ai < 0 || ai >= A) continue;  // not an atom of the model: skipped (the host checks the table)
      const float* Ra = atoms + 3 * ai;
      const float dx = xi[0] - Ra[0], dy = xi[1] - Ra[1], dz = xi[2] - Ra[2];
      const float r = sqrtf(dx * dx + dy * dy + dz * dz);
      // local channel V_0(r)
      const float* tab = radial + ((size_t)a * C + 0) * T * 3;
      for (int t = 0; t < T; ++t) {
        const float al = tab[3 * t], co = tab[3 * t + 1], pw = tab[3 * t + 2];
        if (co != 0.f) loc += co * powf(r, pw) * expf(-al * r * r);
      }
      int pos = MC;
      while (pos > 0 && r < bd[pos - 1]) --pos;
      if (pos < MC) {
        for (int c = MC - 1; c > pos; --c) {
          bd[c] = bd[c - 1];
          best[c] = best[c - 1];
        }
        bd[pos] = r;
        best[pos] = a;
      }
    }
    for (int c = 0; c < MC; ++c) {
      const size_t pr = ((size_t)w * n + i) * MC + c;
      const int a = best[c];
      sel[pr] = a;
      if (a < 0) continue;
      const float* Ra = atoms + 3 * ecp_atoms[a];
      const float r = bd[c];
      rad[pr] = r;
      dir[pr * 3] = (xi[0] - Ra[0]) / r;
      dir[pr * 3 + 1] = (xi[1] - Ra[1]) / r;
      dir[pr * 3 + 2] = (xi[2] - Ra[2]) / r;
      for (int l = 1; l < C; ++l) {
        const float* tab = radial + ((size_t)a * C + l) * T * 3;
        float v = 0.f;
        for (int t = 0; t < T; ++t) {
          const float al = tab[3 * t], co = tab[3 * t + 1], pw = tab[3 * t + 2];
          if (co != 0.f) v += co * powf(r, pw) * expf(-al * r * r);
        }
        vnl[pr * (C - 1) + (l - 1)] = v;
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) loc += __shfl_xor_sync(0xffffffffu, loc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = loc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float s = 0.f;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[k];
    e_local[w] = s;
  }
}

// Displaced configurations of walkers w0 .. w0 + Wc - 1: configuration
// g = ((w n + i) MC + c) Q + q is walker w with electron i moved to
// R + r Rot_i x_q (a copy of the walker when core c was not selected).
__global__ void k_ecp_configs(int Wc, int w0, int n, int MC, int Q, const float* __restrict__ x,
                              const float* __restrict__ atoms, const int* __restrict__ ecp_atoms,
                              const float* __restrict__ quad, const int* __restrict__ sel,
                              const float* __restrict__ dir, const float* __restrict__ rad,
                              const float* __restrict__ rot, float* __restrict__ cfg) {
  const size_t G = (size_t)Wc * n * MC * Q;
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= G * n) return;
  const int j = (int)(e % n);
  const size_t g = e / n;
  const int q = (int)(g % Q);
  const size_t pr = g / Q;  // (local walker, i, c)
  const int c = (int)(pr % MC);
  const int i = (int)((pr / MC) % n);
  const int wl = (int)(pr / ((size_t)MC * n));
  const size_t w = (size_t)w0 + wl;
  const float* xj = x + (w * n + j) * 3;
  float* out = cfg + e * 3;
  const size_t prg = (w * n + i) * MC + c;
  const int a = sel[prg];
  if (j != i || a < 0) {
    out[0] = xj[0];
    out[1] = xj[1];
    out[2] = xj[2];
    return;
  }
  const float* R = rot + (w * n + i) * 9;
  const float* p = quad + 4 * q;
  const float* Ra = atoms + 3 * ecp_atoms[a];
  const float r = rad[prg];
  for (int k = 0; k < 3; ++k) out[k] = Ra[k] + r * (R[3 * k] * p[0] + R[3 * k + 1] * p[1] + R[3 * k + 2] * p[2]);
}

__device__ __forceinline__ float legendre_p(int l, float x) {
  switch (l) {
    case 0: return 1.f;
    case 1: return x;
    case 2: return 0.5f * (3.f * x * x - 1.f);
    default: return 0.5f * (5.f * x * x * x - 3.f * x);
  }
}

// Nonlocal energy of walkers w0 .. w0 + Wc - 1 from the displaced
// configurations' log|psi| and signs: one block per walker.
__global__ void k_ecp_reduce(int w0, int n, int MC, int Q, int L, const float* __restrict__ quad,
                             const int* __restrict__ sel, const float* __restrict__ vnl,
                             const float* __restrict__ dir, const float* __restrict__ rot,
                             const float* __restrict__ lp0, const float* __restrict__ sg0,
                             const float* __restrict__ lp1, const float* __restrict__ sg1, float* __restrict__ e_nl) {
  extern __shared__ float red[];
  const int wl = blockIdx.x;
  const size_t w = (size_t)w0 + wl;
  const float l0 = lp0[w], s0 = sg0[w];
  float acc = 0.f;
  for (int pc = threadIdx.x; pc < n * MC; pc += blockDim.x) {
    const int i = pc / MC;
    const size_t prg = w * n * MC + pc;
    if (sel[prg] < 0) continue;
    const float* R = rot + (w * n + i) * 9;
    const float* u = dir + prg * 3;
    float ch[kEcpMaxChannels - 1] = {0.f, 0.f, 0.f, 0.f};
    for (int q = 0; q < Q; ++q) {
      const float* p = quad + 4 * q;
      const float rx = R[0] * p[0] + R[1] * p[1] + R[2] * p[2];
      const float ry = R[3] * p[0] + R[4] * p[1] + R[5] * p[2];
      const float rz = R[6] * p[0] + R[7] * p[1] + R[8] * p[2];
      const float ct = rx * u[0] + ry * u[1] + rz * u[2];
      const size_t g = ((size_t)wl * n * MC + pc) * Q + q;
      const float ratio = sg1[g] * s0 * expf(lp1[g] - l0);
      for (int l = 0; l < L; ++l) ch[l] += p[3] * legendre_p(l, ct) * ratio;
    }
    for (int l = 0; l < L; ++l) acc += (2.f * l + 1.f) * ch[l] * vnl[prg * L + l];
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float s = 0.f;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[k];
    e_nl[w] = s;
  }
}

static qmc_status model_forward(qmc_model* m, int B, void* ws_fwd, const float* x, float* lp, float* sg,
                                cudaStream_t s) {
  if (m->kind == QMC_KIND_PSIFORMER) return psi_evaluate(m, psi_make_plan(m, B), ws_fwd, x, lp, sg, nullptr, s);
  return evaluate(m, make_plan(m, QMC_OP_FORWARD, B), ws_fwd, x, false, lp, sg, nullptr, nullptr, nullptr, s);
}

}  // namespace qmc

extern "C" size_t qmc_ecp_workspace_size(const qmc_model* m, int batch, int n_channels, int max_core, int n_quad) {
  if (!m || batch < 1 || n_channels < 1 || max_core < 1 || n_quad < 1) return 0;
  return qmc::ecp_shape(m, batch, max_core, n_quad, n_channels - 1).total;
}

extern "C" qmc_status qmc_ecp_energy(qmc_model* m, int batch, const float* electrons, int n_ecp_atoms,
                                     const int* ecp_atoms, int n_channels, int max_terms, const float* radial,
                                     int max_core, int n_quad, const float* quad, const float* rotations,
                                     uint64_t seed, uint64_t counter, float* e_local, float* e_nonlocal, void* ws,
                                     size_t ws_bytes, cudaStream_t s) {
  using namespace qmc;
  if (!m) { set_error("null model"); return QMC_ERR_ARG; }
  if (!m->params_set) { set_error("parameters not set (qmc_model_set_params)"); return QMC_ERR_ARG; }
  if (batch < 1 || !electrons || !ecp_atoms || !radial || !quad || !e_local || !e_nonlocal) {
    set_error("qmc_ecp_energy: bad batch or null array");
    return QMC_ERR_ARG;
  }
  if (n_ecp_atoms < 1 || n_ecp_atoms > m->d.A || n_channels < 1 || n_channels > kEcpMaxChannels ||
      max_terms < 1 || max_core < 1 || max_core > kEcpMaxCore || n_quad < 1 || n_quad > 256) {
    set_error("qmc_ecp_energy: ECP atoms 1..%d, channels 1..%d, max_core 1..%d, quadrature points 1..256",
              m->d.A, kEcpMaxChannels, kEcpMaxCore);
    return QMC_ERR_SHAPE;
  }
  int dev;
  QMC_CUDA(cudaGetDevice(&dev));
  if (dev != m->device) {
    set_error("model lives on device %d but device %d is current", m->device, dev);
    return QMC_ERR_ARG;
  }
  const int L = n_channels - 1;
  const EcpShape e = ecp_shape(m, batch, max_core, n_quad, L);
  if (!ws || ws_bytes < e.total) {
    set_error("workspace too small: %zu bytes given, %zu needed", ws_bytes, e.total);
    return QMC_ERR_WORKSPACE;
  }
  // the model's own forward-pass checks (shapes, precision support) for the
  // largest forward this call makes
  const int g_max = (int)std::max<size_t>((size_t)e.Wc * n_quad * max_core * m->d.n, (size_t)e.Wc);
  QMC_TRY(check_call(m, g_max, at<void>(ws, e.fwd), e.total - e.fwd, QMC_OP_FORWARD));
  const int n = m->d.n;
  const float* atoms = m->arena + m->a.atoms;
  int* sel = at<int>(ws, e.sel);
  float* vnl = at<float>(ws, e.vnl);
  float* dir = at<float>(ws, e.dir);
  float* rad = at<float>(ws, e.rad);
  float* rot = at<float>(ws, e.rot);
  float* lp0 = at<float>(ws, e.lp0);
  float* sg0 = at<float>(ws, e.sg0);
  float* cfg = at<float>(ws, e.cfg);
  float* lp1 = at<float>(ws, e.lp1);
  float* sg1 = at<float>(ws, e.sg1);
  void* fwd = at<void>(ws, e.fwd);
  {
    ProfScope ps_(QMC_KC_OTHER, s);
    const int threads = std::min(256, std::max(32, (n + 31) / 32 * 32));
    k_ecp_prepare<<<batch, threads, (threads / 32) * sizeof(float), s>>>(
        n, m->d.A, n_ecp_atoms, n_channels, max_terms, max_core, electrons, atoms, ecp_atoms, radial, rotations, seed,
        counter, e_local, sel, vnl, dir, rad, rot);
    QMC_CUDA(cudaGetLastError());
  }
  if (L == 0) return cudaMemsetAsync(e_nonlocal, 0, sizeof(float) * batch, s) == cudaSuccess ? QMC_OK : QMC_ERR_CUDA;
  for (int w0 = 0; w0 < batch; w0 += e.Wc) {
    const int Wc = std::min(e.Wc, batch - w0);
    QMC_TRY(model_forward(m, Wc, fwd, electrons + (size_t)w0 * n * 3, lp0 + w0, sg0 + w0, s));
    const size_t G = (size_t)Wc * n * max_core * n_quad;
    {
      ProfScope ps_(QMC_KC_OTHER, s);
      k_ecp_configs<<<(unsigned)((G * n + 255) / 256), 256, 0, s>>>(Wc, w0, n, max_core, n_quad, electrons, atoms,
                                                                    ecp_atoms, quad, sel, dir, rad, rot, cfg);
      QMC_CUDA(cudaGetLastError());
    }
    QMC_TRY(model_forward(m, (int)G, fwd, cfg, lp1, sg1, s));
    {
      ProfScope ps_(QMC_KC_OTHER, s);
      k_ecp_reduce<<<Wc, 128, 4 * sizeof(float), s>>>(w0, n, max_core, n_quad, L, quad, sel, vnl, dir, rot, lp0, sg0,
                                                       lp1, sg1, e_nonlocal);
      QMC_CUDA(cudaGetLastError());
    }
  }
  return QMC_OK;
}
