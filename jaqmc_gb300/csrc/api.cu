// C ABI (include/qmc.h): model arena, workspace planning and the drivers of
// the forward pass, the forward-Laplacian local energy and the MH steps.
#include <stdarg.h>
#include <string.h>

#include <cmath>
#include <string>
#include <type_traits>

#include "common.cuh"
#include "gemm_simt.cuh"
#include "kernels.cuh"
#include "profile.cuh"
#include "plan.cuh"
#include "psiformer.cuh"
#include "stream_tc.cuh"

// Launch `call` as a kernel of profiler class `cls` on stream `s`.
#define QMC_PROF(cls, call)               \
  do {                                    \
    ::qmc::ProfScope ps_((cls), s);       \
    QMC_CUDA(call);                       \
  } while (0)
#define QMC_PROF_TRY(cls, call)           \
  do {                                    \
    ::qmc::ProfScope ps_((cls), s);       \
    QMC_TRY(call);                        \
  } while (0)

namespace qmc {

static thread_local std::string g_err;

void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
}

qmc_status cuda_status(cudaError_t e, const char* what) {
  set_error("CUDA error in %s: %s", what, cudaGetErrorString(e));
  return QMC_ERR_CUDA;
}

// ------------------------------------------------------------ layouts
static qmc_status build_dims(const qmc_ferminet_config* c, Dims* d) {
  memset(d, 0, sizeof *d);
  if (c->n_up < 0 || c->n_down < 0 || c->n_up + c->n_down < 1) {
    set_error("nspins must be non-negative with at least one electron");
    return QMC_ERR_SHAPE;
  }
  d->n_up = c->n_up;
  d->n_dn = c->n_down;
  d->n = c->n_up + c->n_down;
  if (d->n > 64) {
    set_error("at most 64 electrons are supported (got %d)", d->n);
    return QMC_ERR_SHAPE;
  }
  d->A = c->n_atoms;
  if (d->A < 1 || d->A > kMaxAtoms) {
    set_error("n_atoms must be in 1..%d", kMaxAtoms);
    return QMC_ERR_SHAPE;
  }
  d->K = c->ndets;
  if (d->K < 1 || d->K > 64) {
    set_error("ndets must be in 1..64");
    return QMC_ERR_SHAPE;
  }
  d->L = c->n_layers;
  if (d->L < 1 || d->L > QMC_MAX_LAYERS) {
    set_error("n_layers must be in 1..%d", QMC_MAX_LAYERS);
    return QMC_ERR_SHAPE;
  }
  d->C = (d->n_up > 0) + (d->n_dn > 0);
  d->split = c->orbitals_spin_split && d->n_up > 0 && d->n_dn > 0;
  d->env_abs = c->envelope == QMC_ENVELOPE_ABS_ISOTROPIC;
  d->env_kind = c->envelope;
  if (c->envelope < QMC_ENVELOPE_ISOTROPIC || c->envelope > QMC_ENVELOPE_NULL) {
    set_error("unsupported envelope %d", c->envelope);
    return QMC_ERR_UNSUPPORTED;
  }
  int d1 = 4 * d->A, d2 = 4;
  for (int l = 0; l < d->L; ++l) {
    int s = c->hidden_single[l], t = c->hidden_double[l];
    if (s < 8 || s % 8 || s > 1024 || t < 1 || t > 256 || 256 % t) {
      set_error("layer %d: widths (%d, %d) unsupported (single: multiple of 8 up to 1024; "
                "double: a divisor of 256)", l, s, t);
      return QMC_ERR_SHAPE;
    }
    d->d1_in[l] = d1;
    d->d2_in[l] = d2;
    d->d1[l] = s;
    d->d2[l] = t;
    d->upd2[l] = l < d->L - 1;
    d->d1_in_p[l] = round_up(d1, 8);
    d->g1_p[l] = round_up(d->C * d1, 8);
    d->g2_p[l] = round_up(d->C * d2, 8);
    if (l == 0 && d1 == s) {
      set_error("a residual connection on the first layer (4*n_atoms == width) is not supported");
      return QMC_ERR_SHAPE;
    }
    d1 = s;
    if (d->upd2[l]) d2 = t;
  }
  d->d_last = d1;
  d->norb = d->K * d->n;
  d->norb_p = round_up(d->norb, 8);
  return QMC_OK;
}

static void build_param_layout(const Dims& d, ParamLayout* p) {
  size_t o = 0;
  for (int l = 0; l < d.L; ++l) {
    int rows = d.d1_in[l] + d.C * d.d1_in[l] + d.C * d.d2_in[l];
    p->dense1_k[l] = o; o += (size_t)rows * d.d1[l];
    p->dense1_b[l] = o; o += d.d1[l];
    if (d.upd2[l]) {
      p->dense2_k[l] = o; o += (size_t)d.d2_in[l] * d.d2[l];
      p->dense2_b[l] = o; o += d.d2[l];
    }
  }
  int nch = d.split ? 2 : 1;
  for (int s = 0; s < nch; ++s) { p->orb_k[s] = o; o += (size_t)d.d_last * d.norb; }
  for (int s = 0; s < nch; ++s) {
    p->env_pi[s] = o; o += env_pi_floats(d.env_kind, d.n, d.A, d.K);
    p->env_sigma[s] = o; o += env_sigma_floats(d.env_kind, d.n, d.A, d.K);
  }
  p->total = o;
}

static void build_arena(const Dims& d, ArenaLayout* a) {
  size_t o = 0;
  auto take = [&](size_t n) { size_t r = o; o += align_up(n, 64); return r; };
  for (int l = 0; l < d.L; ++l) {
    a->w_main[l] = take((size_t)(d.d1_in_p[l] + d.g2_p[l]) * d.d1[l]);
    a->w_g1[l] = take((size_t)d.g1_p[l] * d.d1[l]);
    a->b1[l] = take(d.d1[l]);
    if (d.upd2[l]) {
      a->w2[l] = take((size_t)d.d2_in[l] * d.d2[l]);
      a->b2[l] = take(d.d2[l]);
    }
  }
  int nch = d.split ? 2 : 1;
  for (int s = 0; s < nch; ++s) a->w_orb[s] = take((size_t)d.d_last * d.norb_p);
  for (int s = 0; s < nch; ++s) {
    a->env_pi[s] = take(env_pi_floats(d.env_kind, d.n, d.A, d.K));
    a->env_sigma[s] = take(env_sigma_floats(d.env_kind, d.n, d.A, d.K));
  }
  a->atoms = take(3 * d.A);
  a->charges = take(d.A);
  for (int l = 0; l < d.L; ++l) {
    a->wt_main[l] = take((size_t)d.d1[l] * (d.d1_in_p[l] + d.g2_p[l]));
    a->wt_g1[l] = take((size_t)d.d1[l] * d.g1_p[l]);
    if (d.upd2[l]) a->wt2[l] = take((size_t)d.d2[l] * d.d2_in[l]);
  }
  for (int s = 0; s < nch; ++s) a->wt_orb[s] = take((size_t)d.norb_p * d.d_last);
  a->k0w = 64 * ((d.d1_in_p[0] + 63) / 64 + (d.g2_p[0] + 63) / 64);
  a->w0_pad = take((size_t)a->k0w * d.d1[0]);
  a->total = o;
  size_t b = 0;
  auto takeb = [&](size_t n) { size_t r = b; b += align_up(n, 128); return r; };
  for (int l = 0; l < d.L; ++l) {  // hi and lo planes of the transposed weights
    a->t_main[l] = takeb(2 * (size_t)d.d1[l] * (d.d1_in_p[l] + d.g2_p[l]));
    a->t_g1[l] = takeb(2 * (size_t)d.d1[l] * d.g1_p[l]);
  }
  for (int s = 0; s < nch; ++s) a->t_orb[s] = takeb(2 * (size_t)d.norb * d.d_last);
  a->t0_pad = takeb(2 * (size_t)d.d1[0] * a->k0w);
  for (int l = 0; l < d.L; ++l) a->pfrag[l] = d.upd2[l] ? takeb(256 * 8) : 0;
  a->total_bf16 = b;
}

// ------------------------------------------------------------ workspace
static int tangent_count(const Dims& d, int op) { return op == QMC_OP_LOCAL_ENERGY ? 3 * d.n + 2 : 1; }

// Padded tangent count: the tensor-core path tiles columns by whole groups
// with a 16-column granularity.
static int padded_tangents(const Dims& d, int T, bool mixed) {
  if (T == 1) return 1;
  return mixed ? tc_padded_tangents(T) : T;
}

double nuclear_repulsion(const float* atoms, const float* charges, int A) {
  double nuc = 0.0;
  for (int I = 0; I < A; ++I)
    for (int J = I + 1; J < A; ++J) {
      double dx = atoms[3 * I] - atoms[3 * J], dy = atoms[3 * I + 1] - atoms[3 * J + 1],
             dz = atoms[3 * I + 2] - atoms[3 * J + 2];
      nuc += (double)charges[I] * charges[J] / std::sqrt(dx * dx + dy * dy + dz * dz);
    }
  return nuc;
}

Plan make_plan(const qmc_model* m, int op, int B) {
  const Dims& d = m->d;
  Plan p{};
  p.B = B;
  p.mixed = m->precision == QMC_PRECISION_MIXED_BF16;
  p.T = tangent_count(d, op);
  p.Tp = padded_tangents(d, p.T, p.mixed);
  p.P2 = p.T > 1 ? 5 : 1;
  p.K0p = d.d1_in_p[0];
  p.act_bytes = 4;
  const size_t rows = (size_t)B * d.n * p.Tp;
  int dmax = 8, g1max = 8, g2max = 8, d2max = 4;
  for (int l = 0; l < d.L; ++l) {
    dmax = std::max(dmax, std::max(d.d1_in_p[l], d.d1[l]));
    g1max = std::max(g1max, d.g1_p[l]);
    g2max = std::max(g2max, d.g2_p[l]);
    d2max = std::max(d2max, d.d2[l]);
  }
  p.dmax = dmax;
  p.g1max = g1max;
  p.g2max = g2max;
  p.h1_plane = rows * dmax;
  p.g1_plane = (size_t)B * p.Tp * g1max;
  p.g2_plane = rows * g2max;
  size_t o = 0;
  auto take = [&](size_t bytes) { size_t r = o; o += align_up(bytes, 256); return r; };
  p.x0 = take(rows * p.K0p * 4);
  // split-bf16 copies of the first layer's operands (mixed form)
  p.x0s = take(p.mixed ? rows * p.K0p * 4 : 0);
  p.g2s0 = take(p.mixed ? rows * d.g2_p[0] * 4 : 0);
  p.h1[0] = take(rows * dmax * p.act_bytes);
  p.h1[1] = take(rows * dmax * p.act_bytes);
  size_t pairs = (size_t)B * d.n * d.n;
  p.h2[0] = take(pairs * p.P2 * d2max * 4);
  p.h2[1] = take(pairs * p.P2 * d2max * 4);
  p.g1 = take((size_t)B * p.Tp * g1max * 4);
  p.gb = take((size_t)B * p.Tp * dmax * 4);
  p.g2 = take(rows * g2max * 4);
  p.rae = take((size_t)B * d.n * d.A * 4);
  p.aevec = take((size_t)B * d.n * d.A * 12);
  p.amat = take((size_t)B * d.K * p.Tp * d.n * d.n * 4);
  p.pe = take((size_t)B * 4);
  p.lpsi = take((size_t)B * 4);
  p.sgn = take((size_t)B * 4);
  p.xp = take((size_t)B * d.n * 12);
  p.lp = take((size_t)B * 4);
  p.refac = take(16);
  p.redo = take(logdet_fl_scratch_bytes(B, d.K, p.T));
  p.total = o;
  return p;
}

template <typename T>
static T* at(void* ws, size_t off) { return reinterpret_cast<T*>(static_cast<char*>(ws) + off); }

// ------------------------------------------------------------ network
// Value-only passes fuse each two-electron layer with the next layer's spin
// means of h2 (and the first layer's means with the features) when the
// widths and the per-walker pair block fit the fused kernel.
static bool pair_fused(const Dims& d, int T) {
  if (T != 1) return false;
  for (int l = 0; l < d.L; ++l) {
    if (!d.upd2[l]) continue;
    const bool w_ok = (d.d2_in[l] == 4 && d.d2[l] == 32) || (d.d2_in[l] == 32 && d.d2[l] == 32);
    if (!w_ok || (size_t)4 * ((size_t)d.n * d.n * d.d2[l] + (size_t)d.d2_in[l] * d.d2[l]) > 200 * 1024)
      return false;
  }
  return true;
}

// Value-only forwards run the whole two-electron stream in one kernel
// (launch_pair_stream_value) when its layers are 32 wide, a walker's pair
// activations fit in shared memory and the per-layer means fit the second
// pair buffer, which that path leaves unused.
static bool pair_stream(const Dims& d, const Plan& p) {
  if (p.T != 1 || d.L < 2 || d.L - 1 > kPairStreamMax) return false;
  for (int l = 0; l < d.L; ++l) {
    if (d.upd2[l] != (l < d.L - 1)) return false;
    if (l < d.L - 1 && (d.d2[l] != 32 || (d.d2_in[l] != 4 && d.d2_in[l] != 32))) return false;
  }
  if (pair_stream_smem(d.n, d.L - 1) > 200 * 1024) return false;
  return (size_t)(d.L - 1) * p.g2_plane * 4 <= p.g1 - p.h2[1];
}

// Mixed passes take every input of the first layer (split features,
// pair-mean rows, broadcast term) from one per-walker kernel: value-only
// passes on the fused two-electron path (launch_inputs_value), tangent passes
// with the compact pair tangents (launch_inputs_fl).
static bool inputs_fused(const Dims& d, const Plan& p) {
  if (!p.mixed) return false;
  if (p.T == 1) return pair_fused(d, p.T) && inputs_value_smem(d.n, d.A, d.g1_p[0]) <= 48 * 1024;
  return p.P2 == 5 && d.d2_in[0] == 4 && inputs_fl_supported(d.n, d.A, p.Tp, d.g1_p[0]);
}

// Tangent passes fuse each two-electron layer with the next one-electron
// layer's pair means (launch_pair_layer_mean_fl) for the widths and electron
// counts that kernel covers.
static bool pair_means_fused(const Dims& d, const Plan& p) {
  if (p.T == 1 || p.P2 != 5 || d.n > 32 || p.T != 3 * d.n + 2) return false;
  for (int l = 0; l < d.L; ++l)
    if (d.upd2[l] && (d.d2[l] != 32 || (d.d2_in[l] != 4 && d.d2_in[l] != 32))) return false;
  return true;
}

// The means after pair layer l - 1 (input of one-electron layer l >= 1) on
// the fused two-electron path: f32 [B*n][g2_p[l]], or two bf16 planes.
static size_t stream_g2(const Plan& p, int l) { return p.h2[1] + (size_t)(l - 1) * p.g2_plane * 4; }

template <class Out>
static qmc_status run_pair_stream(qmc_model* m, const Plan& p, void* ws, cudaStream_t s) {
  const Dims& d = m->d;
  const float* ar = m->arena;
  PairStreamArgs a{};
  PairStreamOut<Out> o{};
  a.n = d.n;
  a.n_up = d.n_up;
  a.C = d.C;
  a.nl = d.L - 1;
  a.H0 = reinterpret_cast<const float*>(static_cast<char*>(ws) + p.h2[0]);
  for (int l = 0; l < a.nl; ++l) {
    a.din[l] = d.d2_in[l];
    a.W[l] = ar + m->a.w2[l];
    a.Wf[l] = reinterpret_cast<const uint4*>(m->arena_bf16 + m->a.pfrag[l]);
    a.b[l] = ar + m->a.b2[l];
    a.g2p[l] = d.g2_p[l + 1];
    char* base = static_cast<char*>(ws) + stream_g2(p, l + 1);
    if constexpr (std::is_same<Out, StSplit>::value) {
      o.G2[l] = StSplit{reinterpret_cast<__nv_bfloat16*>(base), d.g2_p[l + 1], p.g2_plane};
    } else {
      o.G2[l] = StF32{reinterpret_cast<float*>(base), d.g2_p[l + 1]};
    }
  }
  QMC_PROF(QMC_KC_PAIR, launch_pair_stream_value(s, p.B, a, o));
  return QMC_OK;
}

// Plain FP32 form.  One-electron layer l: spin means, broadcast GEMM, main
// GEMM with the tangent epilogue; then the two-electron update.
static qmc_status run_backbone_plain(qmc_model* m, const Plan& p, void* ws, cudaStream_t s, int* out_buf) {
  const Dims& d = m->d;
  const bool fused = pair_fused(d, p.T);
  const bool stream = pair_stream(d, p);
  const bool fl_means = pair_means_fused(d, p);
  if (stream) QMC_TRY(run_pair_stream<StF32>(m, p, ws, s));
  const float* ar = m->arena;
  const ArenaLayout& a = m->a;
  const int B = p.B, Tp = p.Tp, T = p.T, n = d.n;
  const RowMap rows_map{n, 0, n, Tp};
  const RowMap wt_map{1, 0, 1, Tp};
  int cur = 0, h2cur = 0;
  for (int l = 0; l < d.L; ++l) {
    const int din = d.d1_in[l], dinp = d.d1_in_p[l], dout = d.d1[l];
    const float* in = l == 0 ? at<float>(ws, p.x0) : at<float>(ws, p.h1[cur]);
    float* out = at<float>(ws, p.h1[l == 0 ? 0 : cur ^ 1]);
    float* G1 = at<float>(ws, p.g1);
    float* Gb = at<float>(ws, p.gb);
    float* G2 = at<float>(ws, stream && l > 0 ? stream_g2(p, l) : p.g2);
    const float* H2 = at<float>(ws, p.h2[h2cur]);
    QMC_PROF(QMC_KC_MEANS, launch_mean_h1(s, B, n, d.n_up, d.C, Tp, din, StF32{const_cast<float*>(in), dinp},
                                          d.g1_p[l], StF32{G1, d.g1_p[l]}));
    QMC_PROF(QMC_KC_BROADCAST, launch_gemm_simt(s, B, wt_map, G1, d.g1_p[l], d.g1_p[l], nullptr, 0, 0,
                                                ar + a.w_g1[l], dout, dout, EpiStore{Gb, dout, nullptr}));
    if (!fused && !stream && !(l > 0 && fl_means))
      QMC_PROF(QMC_KC_MEANS, launch_mean_h2(s, B, n, d.n_up, d.C, Tp, T, d.d2_in[l], p.P2, H2, d.g2_p[l],
                                            StF32{G2, d.g2_p[l]}));
    EpiLayer<StF32> epi{Gb, ar + a.b1[l], StF32{nullptr, dout}, StF32{out, dout}, T};
    if (l > 0 && din == dout) epi.resid = StF32{const_cast<float*>(in), dout};
    QMC_PROF(l == 0 ? QMC_KC_LAYER0 : QMC_KC_STREAM_LAYER,
             launch_gemm_simt(s, B * n, rows_map, in, dinp, dinp, G2, d.g2_p[l], d.g2_p[l], ar + a.w_main[l], dout,
                              dout, epi));
    if (d.upd2[l] && !stream) {
      float* h2o = at<float>(ws, p.h2[h2cur ^ 1]);
      if (fused)
        QMC_PROF(QMC_KC_PAIR, launch_pair_layer_mean(s, B, n, d.n_up, d.C, d.d2_in[l], d.d2[l], H2, ar + a.w2[l],
                                                     ar + a.b2[l], h2o, d.g2_p[l + 1], StF32{G2, d.g2_p[l + 1]}));
      else if (fl_means)  // the pair output is read again only by a later pair layer
        QMC_PROF(QMC_KC_PAIR,
                 launch_pair_layer_mean_fl(s, B, n, d.n_up, d.C, Tp, T, d.d2_in[l], d.d2[l], H2, ar + a.w2[l],
                                           ar + a.b2[l], d.upd2[l + 1] ? h2o : nullptr, d.g2_p[l + 1],
                                           StF32{at<float>(ws, p.g2), d.g2_p[l + 1]}));
      else
        QMC_PROF(QMC_KC_PAIR, launch_pair_layer(s, B * n * n, p.P2, d.d2_in[l], d.d2[l], H2, ar + a.w2[l],
                                                ar + a.b2[l], h2o));
      h2cur ^= 1;
    }
    cur = (l == 0) ? 0 : cur ^ 1;
  }
  *out_buf = cur;
  return QMC_OK;
}

// Mixed form: the first layer (4A-wide input) in FP32; every later layer,
// its broadcast term and the orbitals as split-BF16 tcgen05 GEMMs.
static qmc_status run_backbone_mixed(qmc_model* m, const Plan& p, void* ws, cudaStream_t s, int* out_buf) {
  const Dims& d = m->d;
  const bool fused = pair_fused(d, p.T);
  const bool stream = pair_stream(d, p);
  const bool fl_means = pair_means_fused(d, p);
  if (stream) QMC_TRY(run_pair_stream<StSplit>(m, p, ws, s));
  const float* ar = m->arena;
  const ArenaLayout& a = m->a;
  const int B = p.B, Tp = p.Tp, T = p.T, n = d.n;
  const RowMap rows_map{n, 0, n, Tp};
  const RowMap wt_map{1, 0, 1, Tp};
  typedef __nv_bfloat16 bf;
  int cur = 0, h2cur = 0;
  for (int l = 0; l < d.L; ++l) {
    const int din = d.d1_in[l], dinp = d.d1_in_p[l], dout = d.d1[l];
    bf* out = at<bf>(ws, p.h1[l == 0 ? 0 : cur ^ 1]);
    float* Gb = at<float>(ws, p.gb);
    const float* H2 = at<float>(ws, p.h2[h2cur]);
    if (l == 0) {
      // first layer (4A-wide features): spin means and broadcast term in FP32,
      // the main GEMM on the tensor cores from split-bf16 copies of the
      // features and pair means, with the chunk-padded kernel
      float* X0 = at<float>(ws, p.x0);
      float* G1 = at<float>(ws, p.g1);
      const size_t rows = (size_t)B * n * Tp;
      bf* X0s = at<bf>(ws, p.x0s);
      bf* G2s = at<bf>(ws, p.g2s0);
      if (!inputs_fused(d, p)) {  // else evaluate() wrote X0s, G2s and Gb
        QMC_PROF(QMC_KC_MEANS, launch_mean_h1(s, B, n, d.n_up, d.C, Tp, din, StF32{X0, dinp}, d.g1_p[l],
                                              StF32{G1, d.g1_p[l]}));
        QMC_PROF(QMC_KC_BROADCAST, launch_gemm_simt(s, B, wt_map, G1, d.g1_p[l], d.g1_p[l], nullptr, 0, 0,
                                                    ar + a.w_g1[l], dout, dout, EpiStore{Gb, dout, nullptr}));
        if (!fused)
          QMC_PROF(QMC_KC_MEANS, launch_mean_h2(s, B, n, d.n_up, d.C, Tp, T, d.d2_in[l], p.P2, H2, d.g2_p[l],
                                                StSplit{G2s, d.g2_p[l], rows * d.g2_p[l]}));
        else
          QMC_PROF(QMC_KC_LAYER0,
                   launch_to_split(s, rows * d.g2_p[l], at<float>(ws, p.g2), G2s, rows * d.g2_p[l]));
        QMC_PROF(QMC_KC_LAYER0, launch_to_split(s, rows * dinp, X0, X0s, rows * dinp));
      }
      TcLayerArgs la{};
      la.n_groups = B * n;
      la.n = n;
      la.Tp = Tp;
      la.T = T;
      la.X = X0s;
      la.k1 = dinp;
      la.x_plane = rows * dinp;
      la.G2 = G2s;
      la.k2 = d.g2_p[l];
      la.g2_plane = rows * d.g2_p[l];
      la.Wt = m->arena_bf16 + a.t0_pad;
      la.w_ld = a.k0w;
      la.n_out = dout;
      la.Gb = Gb;
      la.bias = ar + a.b1[l];
      la.residual = false;
      la.out = out;
      la.out_plane = p.h1_plane;
      la.err = m->dev_err;
      QMC_PROF_TRY(QMC_KC_LAYER0, tc_stream_layer(s, la));
    } else {
      bf* in = at<bf>(ws, p.h1[cur]);
      bf* G1 = at<bf>(ws, p.g1);
      bf* G2 = at<bf>(ws, stream ? stream_g2(p, l) : p.g2);
      const int kmain = dinp + d.g2_p[l];
      QMC_PROF(QMC_KC_MEANS, launch_mean_h1(s, B, n, d.n_up, d.C, Tp, din, StSplit{in, dinp, p.h1_plane},
                                            d.g1_p[l], StSplit{G1, d.g1_p[l], p.g1_plane}));
      TcStoreArgs sa{B * Tp, G1, d.g1_p[l], p.g1_plane, m->arena_bf16 + a.t_g1[l], dout, Gb, m->dev_err};
      QMC_PROF_TRY(QMC_KC_BROADCAST, tc_store_gemm(s, sa));
      if (!fused && !stream && !fl_means)
        QMC_PROF(QMC_KC_MEANS, launch_mean_h2(s, B, n, d.n_up, d.C, Tp, T, d.d2_in[l], p.P2, H2, d.g2_p[l],
                                              StSplit{G2, d.g2_p[l], p.g2_plane}));
      TcLayerArgs la{};
      la.n_groups = B * n;
      la.n = n;
      la.Tp = Tp;
      la.T = T;
      la.X = in;
      la.k1 = dinp;
      la.x_plane = p.h1_plane;
      la.G2 = G2;
      la.k2 = d.g2_p[l];
      la.g2_plane = p.g2_plane;
      la.Wt = m->arena_bf16 + a.t_main[l];
      la.n_out = dout;
      la.Gb = Gb;
      la.bias = ar + a.b1[l];
      la.residual = din == dout;
      la.out = out;
      la.out_plane = p.h1_plane;
      la.err = m->dev_err;
      (void)kmain;
      QMC_PROF_TRY(QMC_KC_STREAM_LAYER, tc_stream_layer(s, la));
    }
    if (d.upd2[l] && !stream) {
      float* h2o = at<float>(ws, p.h2[h2cur ^ 1]);
      if (fused)  // next layer (>= 1) reads its G2 as split bf16
        QMC_PROF(QMC_KC_PAIR, launch_pair_layer_mean(s, B, n, d.n_up, d.C, d.d2_in[l], d.d2[l], H2, ar + a.w2[l],
                                                     ar + a.b2[l], h2o, d.g2_p[l + 1],
                                                     StSplit{at<bf>(ws, p.g2), d.g2_p[l + 1], p.g2_plane}));
      else if (fl_means)  // the pair output is read again only by a later pair layer
        QMC_PROF(QMC_KC_PAIR,
                 launch_pair_layer_mean_fl(s, B, n, d.n_up, d.C, Tp, T, d.d2_in[l], d.d2[l], H2, ar + a.w2[l],
                                           ar + a.b2[l], d.upd2[l + 1] ? h2o : nullptr, d.g2_p[l + 1],
                                           StSplit{at<bf>(ws, p.g2), d.g2_p[l + 1], p.g2_plane}));
      else
        QMC_PROF(QMC_KC_PAIR, launch_pair_layer(s, B * n * n, p.P2, d.d2_in[l], d.d2[l], H2, ar + a.w2[l],
                                                ar + a.b2[l], h2o));
      h2cur ^= 1;
    }
    cur = (l == 0) ? 0 : cur ^ 1;
  }
  *out_buf = cur;
  return QMC_OK;
}

// Value-only mixed passes take the envelope factor out of the tensor-core
// epilogue (too few warps to hide its exponentials): a full-occupancy kernel
// writes the factors into the two-electron buffer, unused by then, and the LU
// kernel multiplies them in as it loads the matrices.
static bool env_in_lu(const Dims& d, const Plan& p) {
  const bool params_fit = (size_t)8 * (d.split ? 2 : 1) * d.A * d.K * d.n <= 48 * 1024;
  return p.mixed && p.T == 1 && d.n <= 32 && params_fit &&
         p.h2[1] - p.h2[0] >= (size_t)p.B * d.K * d.n * d.n * sizeof(float);
}

// Where the value-only mixed passes apply the envelope: 1 = factors from
// launch_envelope_value multiplied in by the register LU (n <= 32), 2 = raw
// orbitals multiplied in place by launch_envelope_apply before the LU;
// 0 = inside the orbital epilogue (FP32 form and tangent passes).
static int env_mode(const Dims& d, const Plan& p) {
  if (!p.mixed || p.T != 1 || !env_in_epilogue(d.env_kind)) return 0;
  if (env_in_lu(d, p)) return 1;
  const bool fits = (size_t)4 * (2 * (d.split ? 2 : 1) * d.A * d.n + d.n * d.A) <= 48 * 1024;
  return d.n <= 64 && fits ? 2 : 0;
}

// The diagonal envelope, after an orbital stage that stored the orbitals
// without one (nothing to do for the other envelopes).
static qmc_status apply_late_envelope(qmc_model* m, const Plan& p, void* ws, cudaStream_t s) {
  const Dims& d = m->d;
  if (d.env_kind != QMC_ENVELOPE_DIAGONAL) return QMC_OK;
  const float* ar = m->arena;
  const int c1 = d.split ? 1 : 0;
  QMC_PROF(QMC_KC_ORBITAL, launch_envelope_diag(s, p.B, d.n, d.n_up, d.split, d.K, d.A, p.Tp, p.T,
                                                ar + m->a.env_pi[0], ar + m->a.env_sigma[0], ar + m->a.env_pi[c1],
                                                ar + m->a.env_sigma[c1], at<float>(ws, p.aevec),
                                                at<float>(ws, p.amat)));
  return QMC_OK;
}

qmc_status run_orbitals(qmc_model* m, const Plan& p, void* ws, int hb, cudaStream_t s) {
  const Dims& d = m->d;
  const ArenaLayout& a = m->a;
  const float* ar = m->arena;
  int nch = d.split ? 2 : 1;
  if (p.mixed) {
    TcOrbitalArgs oa{};
    oa.B = p.B;
    oa.n = d.n;
    oa.n_up = d.n_up;
    oa.split = d.split;
    oa.Tp = p.Tp;
    oa.T = p.T;
    oa.K = d.K;
    oa.natom = d.A;
    oa.env_abs = d.env_abs;
    oa.X = at<__nv_bfloat16>(ws, p.h1[hb]);
    oa.k = d.d_last;
    oa.x_plane = p.h1_plane;
    for (int c = 0; c < 2; ++c) {
      int cc = c < nch ? c : 0;
      oa.Wt[c] = m->arena_bf16 + a.t_orb[cc];
      oa.pi[c] = ar + a.env_pi[cc];
      oa.sigma[c] = ar + a.env_sigma[cc];
    }
    oa.norb = d.norb;
    oa.rae = at<float>(ws, p.rae);
    oa.aevec = at<float>(ws, p.aevec);
    oa.A = at<float>(ws, p.amat);
    const bool epi_env = env_in_epilogue(d.env_kind);
    oa.raw = epi_env ? env_mode(d, p) != 0 : 1;
    oa.unit_env = !epi_env;
    oa.err = m->dev_err;
    QMC_PROF_TRY(QMC_KC_ORBITAL, tc_orbitals(s, oa));
    return apply_late_envelope(m, p, ws, s);
  }
  const float* h = at<float>(ws, p.h1[hb]);
  for (int c = 0; c < nch; ++c) {
    int ns = d.split ? (c == 0 ? d.n_up : d.n_dn) : d.n;
    int i0 = (d.split && c == 1) ? d.n_up : 0;
    RowMap map{ns, i0, d.n, p.Tp};
    EpiOrbital epi{at<float>(ws, p.amat), at<float>(ws, p.rae), at<float>(ws, p.aevec),
                   ar + a.env_pi[c], ar + a.env_sigma[c], d.n, d.A, d.K, p.T, d.env_abs};
    epi.unit_env = !env_in_epilogue(d.env_kind);
    QMC_PROF(QMC_KC_ORBITAL, launch_gemm_simt(s, p.B * ns, map, h, d.d_last, d.d_last, nullptr, 0, 0,
                                              ar + a.w_orb[c], d.norb_p, d.norb, epi));
  }
  return apply_late_envelope(m, p, ws, s);
}

// Determinant stage: LU (with the value-only envelope factors when the
// orbital epilogue left them out), log-sum-exp, and for tangent passes the
// kinetic and local energy.
qmc_status run_logdet(qmc_model* m, const Plan& p, void* ws, const float* pe, float* logpsi, float* sign,
                      float* ke, float* el, uint8_t* flags, cudaStream_t s) {
  const Dims& d = m->d;
  const float* ar = m->arena;
  EnvArgs env{};
  const int mode = env_mode(d, p);
  const int c1 = d.split ? 1 : 0;
  if (mode == 1) {
    env.env = at<float>(ws, p.h2[0]);
    QMC_PROF(QMC_KC_ORBITAL, launch_envelope_value(s, p.B, d.n, d.n_up, d.split, d.K, d.A, d.env_abs,
                                                   ar + m->a.env_pi[0], ar + m->a.env_sigma[0],
                                                   ar + m->a.env_pi[c1], ar + m->a.env_sigma[c1],
                                                   at<float>(ws, p.rae), const_cast<float*>(env.env)));
  } else if (mode == 2) {
    QMC_PROF(QMC_KC_ORBITAL, launch_envelope_apply(s, p.B, d.n, d.n_up, d.split, d.K, d.A, d.env_abs,
                                                   ar + m->a.env_pi[0], ar + m->a.env_sigma[0],
                                                   ar + m->a.env_pi[c1], ar + m->a.env_sigma[c1],
                                                   at<float>(ws, p.rae), at<float>(ws, p.amat)));
  }
  QMC_PROF(QMC_KC_LOGDET, launch_logdet(s, p.B, d.n, d.K, p.Tp, p.T, at<float>(ws, p.amat), pe, logpsi, sign, ke, el,
                                        flags, nullptr, mode == 1 ? &env : nullptr, nullptr,
                                        at<void>(ws, p.redo), m->det_guard_on()));
  return QMC_OK;
}

// Full evaluation: features -> backbone -> orbitals -> determinants.
qmc_status evaluate(qmc_model* m, const Plan& p, void* ws, const float* electrons, bool want_pe,
                           float* logpsi, float* sign, float* ke, float* el, uint8_t* flags,
                           cudaStream_t s) {
  if (m->kind != QMC_KIND_FERMINET) {
    set_error("this entry point evaluates FermiNet models only");
    return QMC_ERR_UNSUPPORTED;
  }
  const Dims& d = m->d;
  const float* ar = m->arena;
  float* pe = want_pe ? at<float>(ws, p.pe) : nullptr;
  const bool fused = pair_fused(d, p.T);
  if (inputs_fused(d, p)) {
    typedef __nv_bfloat16 bf;
    const size_t rows = (size_t)p.B * d.n * p.Tp;
    const StSplit x0s{at<bf>(ws, p.x0s), p.K0p, rows * p.K0p};
    const StSplit g2s{at<bf>(ws, p.g2s0), d.g2_p[0], rows * d.g2_p[0]};
    if (p.T == 1)
      QMC_PROF(QMC_KC_FEATURES,
               launch_inputs_value(s, p.B, d.n, d.A, d.n_up, d.C, p.K0p, d.g1_p[0], d.g2_p[0], d.d1[0], electrons,
                                   ar + m->a.atoms, ar + m->a.charges, m->nuclear_repulsion, ar + m->a.w_g1[0],
                                   at<float>(ws, p.rae), at<float>(ws, p.aevec), at<float>(ws, p.h2[0]), x0s, g2s,
                                   at<float>(ws, p.gb), pe));
    else
      QMC_PROF(QMC_KC_FEATURES,
               launch_inputs_fl(s, p.B, d.n, d.A, d.n_up, d.C, p.Tp, p.T, p.K0p, d.g1_p[0], d.g2_p[0], d.d1[0],
                                electrons, ar + m->a.atoms, ar + m->a.charges, m->nuclear_repulsion,
                                ar + m->a.w_g1[0], at<float>(ws, p.rae), at<float>(ws, p.aevec),
                                at<float>(ws, p.h2[0]), x0s, g2s, at<float>(ws, p.gb), pe));
  } else {
    QMC_PROF(QMC_KC_FEATURES, launch_features(s, p.B, d.n, d.A, p.Tp, p.T, p.K0p, electrons, ar + m->a.atoms,
                                              ar + m->a.charges, m->nuclear_repulsion, at<float>(ws, p.x0),
                                              at<float>(ws, p.h2[0]), at<float>(ws, p.rae), at<float>(ws, p.aevec),
                                              pe, d.n_up, d.C, d.g2_p[0], fused ? at<float>(ws, p.g2) : nullptr));
  }
  int hb = 0;
  if (p.mixed) QMC_TRY(run_backbone_mixed(m, p, ws, s, &hb));
  else QMC_TRY(run_backbone_plain(m, p, ws, s, &hb));
  QMC_TRY(run_orbitals(m, p, ws, hb, s));
  return run_logdet(m, p, ws, pe, logpsi, sign, ke, el, flags, s);
}

qmc_status check_call(qmc_model* m, int batch, const void* ws, size_t ws_bytes, int op) {
  if (!m) { set_error("null model"); return QMC_ERR_ARG; }
  if (!m->params_set) { set_error("parameters not set (qmc_model_set_params)"); return QMC_ERR_ARG; }
  if (batch < 1) { set_error("batch must be >= 1"); return QMC_ERR_SHAPE; }
  if (m->kind == QMC_KIND_PSIFORMER) {
    if (op != QMC_OP_FORWARD && op != QMC_OP_MH && op != QMC_OP_LOCAL_ENERGY) {
      set_error("attention-backbone models take qmc_forward, MH steps and the local energy here (the Psiformer adjoint is qmc_grad)");
      return QMC_ERR_UNSUPPORTED;
    }
    if (op == QMC_OP_LOCAL_ENERGY) QMC_TRY(psi_fl_check(m));
    const size_t need = op == QMC_OP_LOCAL_ENERGY ? psi_fl_plan(m, psi_fl_chunk(m, batch)).base.total
                                                  : psi_make_plan(m, batch).base.total;
    if (!ws || ws_bytes < need) {
      set_error("workspace too small: %zu bytes given, %zu needed", ws_bytes, need);
      return QMC_ERR_WORKSPACE;
    }
    int dev;
    QMC_CUDA(cudaGetDevice(&dev));
    if (dev != m->device) {
      set_error("model lives on device %d but device %d is current", m->device, dev);
      return QMC_ERR_ARG;
    }
    return QMC_OK;
  }
  if (m->precision == QMC_PRECISION_MIXED_BF16) {
    const Dims& d = m->d;
    for (int l = 1; l < d.L; ++l)
      if (d.d1_in_p[l] % 64 || !tc_layer_supported(d.d1_in_p[l], d.g2_p[l], d.d1[l])) {
        set_error("mixed precision needs one-electron widths that are multiples of 64 (layer %d)", l);
        return QMC_ERR_UNSUPPORTED;
      }
    if (d.d_last % 64 || make_plan(m, op, 1).Tp < 0) {
      set_error("mixed precision needs a last width that is a multiple of 64");
      return QMC_ERR_UNSUPPORTED;
    }
  }
  if (op == QMC_OP_LOCAL_ENERGY && make_plan(m, op, 1).Tp > 128) {
    set_error("local energy supports at most 42 electrons (3n+2 <= 128 tangents per tile)");
    return QMC_ERR_SHAPE;
  }
  size_t need = make_plan(m, op, batch).total;
  if (!ws || ws_bytes < need) {
    set_error("workspace too small: %zu bytes given, %zu needed", ws_bytes, need);
    return QMC_ERR_WORKSPACE;
  }
  int dev;
  QMC_CUDA(cudaGetDevice(&dev));
  if (dev != m->device) {
    set_error("model lives on device %d but device %d is current", m->device, dev);
    return QMC_ERR_ARG;
  }
  return QMC_OK;
}

// Body of qmc_mh_steps / qmc_mh_steps_resident: the update index of step st is
// counter + st (+ *ctr_dev when ctr_dev is set).
qmc_status mh_steps(qmc_model* m, int batch, int steps, float stddev, uint64_t seed, uint64_t counter,
                    const uint64_t* ctr_dev, float* electrons, float* log_prob, uint32_t* accepts,
                    const float* inj_normals, const float* inj_uniforms, uint8_t* flags, void* ws,
                    size_t ws_bytes, cudaStream_t s, const MhGroup& grp = MhGroup{}) {
  QMC_TRY(check_call(m, batch, ws, ws_bytes, QMC_OP_MH));
  if (!electrons || !log_prob || steps < 0) { set_error("bad electrons/log_prob/steps"); return QMC_ERR_ARG; }
  const bool psi = m->kind == QMC_KIND_PSIFORMER;
  const PsiPlan pp = psi ? psi_make_plan(m, batch) : PsiPlan{};
  const Plan p = psi ? pp.base : make_plan(m, QMC_OP_MH, batch);
  auto forward = [&](const float* x, float* lp, uint8_t* fl) -> qmc_status {
    if (psi) return psi_evaluate(m, pp, ws, x, lp, at<float>(ws, p.sgn), fl, s);
    return evaluate(m, p, ws, x, false, lp, at<float>(ws, p.sgn), nullptr, nullptr, fl, s);
  };
  const int n = m->d.n;
  float* lpsi = at<float>(ws, p.lpsi);
  // log_prob of the starting walkers (src/jaqmc/sampler/mcmc.py:166)
  QMC_TRY(forward(electrons, lpsi, flags));
  QMC_PROF(QMC_KC_OTHER, launch_scale(s, batch, lpsi, 2.0f, log_prob));
  float* xp = at<float>(ws, p.xp);
  for (int st = 0; st < steps; ++st) {
    const float* nz = inj_normals ? inj_normals + (size_t)st * batch * n * 3 : nullptr;
    const float* uz = inj_uniforms ? inj_uniforms + (size_t)st * batch : nullptr;
    QMC_PROF(QMC_KC_MH,
             launch_mh_propose(s, batch, n, electrons, xp, stddev, seed, counter + st, ctr_dev, nz, grp));
    QMC_TRY(forward(xp, lpsi, nullptr));
    QMC_PROF(QMC_KC_MH, launch_mh_accept(s, batch, n, electrons, xp, log_prob, lpsi, seed, counter + st, ctr_dev,
                                         uz, accepts, grp));
  }
  return QMC_OK;
}

}  // namespace qmc

using namespace qmc;

extern "C" {

const char* qmc_last_error(void) { return qmc::g_err.c_str(); }

qmc_status qmc_device_check(int* major, int* minor, int* n_sms) {
  int dev;
  QMC_CUDA(cudaGetDevice(&dev));
  cudaDeviceProp pr;
  QMC_CUDA(cudaGetDeviceProperties(&pr, dev));
  if (major) *major = pr.major;
  if (minor) *minor = pr.minor;
  if (n_sms) *n_sms = pr.multiProcessorCount;
  if (!(pr.major == 10 && pr.minor == 3)) {
    set_error("device %s is sm_%d%d; this library is built for sm_103a", pr.name, pr.major, pr.minor);
    return QMC_ERR_UNSUPPORTED;
  }
  return QMC_OK;
}

qmc_status qmc_ferminet_create(const qmc_ferminet_config* cfg, const float* atoms_host,
                               const float* charges_host, qmc_model** out) {
  if (!cfg || !atoms_host || !charges_host || !out) {
    set_error("null argument");
    return QMC_ERR_ARG;
  }
  *out = nullptr;
  qmc_model* m = new qmc_model();
  qmc_status st = build_dims(cfg, &m->d);
  if (st != QMC_OK) { delete m; return st; }
  if (cfg->precision != QMC_PRECISION_FP32 && cfg->precision != QMC_PRECISION_MIXED_BF16) {
    delete m;
    set_error("unknown precision %d", cfg->precision);
    return QMC_ERR_ARG;
  }
  m->precision = cfg->precision;
  build_param_layout(m->d, &m->p);
  build_arena(m->d, &m->a);
  cudaError_t e = cudaGetDevice(&m->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&m->n_sms, cudaDevAttrMultiProcessorCount, m->device);
  if (e == cudaSuccess) e = cudaMalloc(&m->arena, m->a.total * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->arena_bf16, m->a.total_bf16 * sizeof(__nv_bfloat16));
  if (e == cudaSuccess) e = cudaMalloc(&m->dev_err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(m->dev_err, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(m->arena, 0, m->a.total * sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(m->arena_bf16, 0, m->a.total_bf16 * sizeof(__nv_bfloat16));
  const int A = m->d.A;
  memcpy(m->atoms_host, atoms_host, sizeof(float) * 3 * A);
  memcpy(m->charges_host, charges_host, sizeof(float) * A);
  m->nuclear_repulsion = nuclear_repulsion(atoms_host, charges_host, A);
  if (e == cudaSuccess)
    e = cudaMemcpy(m->arena + m->a.atoms, atoms_host, sizeof(float) * 3 * A, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(m->arena + m->a.charges, charges_host, sizeof(float) * A, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(m->arena);
    cudaFree(m->arena_bf16);
    cudaFree(m->dev_err);
    delete m;
    return cuda_status(e, "qmc_ferminet_create");
  }
  *out = m;
  return QMC_OK;
}

qmc_status qmc_model_destroy(qmc_model* m) {
  if (!m) return QMC_OK;
  delete m->psi;
  cudaFree(m->arena);
  cudaFree(m->arena_bf16);
  cudaFree(m->dev_err);
  delete m;
  return QMC_OK;
}

qmc_status qmc_model_check_error(qmc_model* m, int* code) {
  if (!m || !code) { set_error("null argument"); return QMC_ERR_ARG; }
  QMC_CUDA(cudaMemcpy(code, m->dev_err, sizeof(int), cudaMemcpyDeviceToHost));
  QMC_CUDA(cudaMemset(m->dev_err, 0, sizeof(int)));
  if (*code) {
    set_error("a bounded device-side wait expired (code %d)", *code);
    return QMC_ERR_TIMEOUT;
  }
  return QMC_OK;
}

size_t qmc_param_count(const qmc_model* m) {
  if (!m) return 0;
  return m->kind == QMC_KIND_PSIFORMER ? m->psi->p.total : m->p.total;
}

qmc_status qmc_model_set_precision(qmc_model* m, int precision) {
  if (!m) { set_error("null model"); return QMC_ERR_ARG; }
  if (precision != QMC_PRECISION_FP32 && precision != QMC_PRECISION_MIXED_BF16) {
    set_error("unknown precision %d", precision);
    return QMC_ERR_ARG;
  }
  m->precision = precision;
  return QMC_OK;
}

qmc_status qmc_model_set_params(qmc_model* m, const float* params, cudaStream_t s) {
  if (!m || !params) { set_error("null argument"); return QMC_ERR_ARG; }
  if (m->kind == QMC_KIND_PSIFORMER) return psi_set_params(m, params, s);
  const Dims& d = m->d;
  const ArenaLayout& a = m->a;
  const ParamLayout& p = m->p;
  float* ar = m->arena;
  auto cp = [&](size_t dst, size_t src, size_t count) {
    return cudaMemcpyAsync(ar + dst, params + src, count * sizeof(float), cudaMemcpyDeviceToDevice, s);
  };
  for (int l = 0; l < d.L; ++l) {
    const int din = d.d1_in[l], dout = d.d1[l];
    QMC_CUDA(cudaMemsetAsync(ar + a.w_main[l], 0, sizeof(float) * (d.d1_in_p[l] + d.g2_p[l]) * dout, s));
    QMC_CUDA(cudaMemsetAsync(ar + a.w_g1[l], 0, sizeof(float) * d.g1_p[l] * dout, s));
    size_t k = p.dense1_k[l];
    // rows [h1 | g1 (C*din) | g2 (C*d2in)] of the reference kernel
    QMC_CUDA(cp(a.w_main[l], k, (size_t)din * dout));
    QMC_CUDA(cp(a.w_g1[l], k + (size_t)din * dout, (size_t)d.C * din * dout));
    QMC_CUDA(cp(a.w_main[l] + (size_t)d.d1_in_p[l] * dout, k + (size_t)(din + d.C * din) * dout,
                (size_t)d.C * d.d2_in[l] * dout));
    QMC_CUDA(cp(a.b1[l], p.dense1_b[l], dout));
    if (d.upd2[l]) {
      QMC_CUDA(cp(a.w2[l], p.dense2_k[l], (size_t)d.d2_in[l] * d.d2[l]));
      QMC_CUDA(cp(a.b2[l], p.dense2_b[l], d.d2[l]));
    }
  }
  int nch = d.split ? 2 : 1;
  for (int c = 0; c < nch; ++c) {
    QMC_CUDA(cudaMemsetAsync(ar + a.w_orb[c], 0, sizeof(float) * d.d_last * d.norb_p, s));
    QMC_CUDA(cudaMemcpy2DAsync(ar + a.w_orb[c], sizeof(float) * d.norb_p, params + p.orb_k[c],
                               sizeof(float) * d.norb, sizeof(float) * d.norb, d.d_last,
                               cudaMemcpyDeviceToDevice, s));
    if (d.env_kind != QMC_ENVELOPE_NULL) {
      QMC_CUDA(cp(a.env_pi[c], p.env_pi[c], env_pi_floats(d.env_kind, d.n, d.A, d.K)));
      QMC_CUDA(cp(a.env_sigma[c], p.env_sigma[c], env_sigma_floats(d.env_kind, d.n, d.A, d.K)));
    }
  }
  // FP32 transposes for the adjoint
  for (int l = 0; l < d.L; ++l) {
    const int kmain = d.d1_in_p[l] + d.g2_p[l];
    QMC_CUDA(launch_transpose_f32(s, ar + a.w_main[l], kmain, d.d1[l], d.d1[l], ar + a.wt_main[l]));
    QMC_CUDA(launch_transpose_f32(s, ar + a.w_g1[l], d.g1_p[l], d.d1[l], d.d1[l], ar + a.wt_g1[l]));
    if (d.upd2[l]) QMC_CUDA(launch_transpose_f32(s, ar + a.w2[l], d.d2_in[l], d.d2[l], d.d2[l], ar + a.wt2[l]));
  }
  for (int c = 0; c < nch; ++c) {
    QMC_CUDA(cudaMemsetAsync(ar + a.wt_orb[c], 0, sizeof(float) * d.norb_p * d.d_last, s));
    QMC_CUDA(launch_transpose_f32(s, ar + a.w_orb[c], d.d_last, d.norb, d.norb_p, ar + a.wt_orb[c]));
  }
  // bf16 K-major copies for the tensor-core path
  for (int l = 0; l < d.L; ++l) {
    int kmain = d.d1_in_p[l] + d.g2_p[l];
    QMC_CUDA(launch_transpose_split(s, ar + a.w_main[l], kmain, d.d1[l], d.d1[l],
                                    m->arena_bf16 + a.t_main[l], kmain, d.d1[l]));
    QMC_CUDA(launch_transpose_split(s, ar + a.w_g1[l], d.g1_p[l], d.d1[l], d.d1[l],
                                    m->arena_bf16 + a.t_g1[l], d.g1_p[l], d.d1[l]));
  }
  for (int c = 0; c < nch; ++c)
    QMC_CUDA(launch_transpose_split(s, ar + a.w_orb[c], d.d_last, d.norb, d.norb_p,
                                    m->arena_bf16 + a.t_orb[c], d.d_last, d.norb));
  // first-layer kernel with per-source chunk padding: feature rows at 0,
  // pair-mean rows at the next multiple of 64
  {
    const int d1 = d.d1[0], kx = d.d1_in_p[0], k2 = d.g2_p[0], o2 = 64 * ((kx + 63) / 64);
    QMC_CUDA(cudaMemsetAsync(ar + a.w0_pad, 0, sizeof(float) * a.k0w * d1, s));
    QMC_CUDA(cudaMemcpyAsync(ar + a.w0_pad, ar + a.w_main[0], sizeof(float) * kx * d1, cudaMemcpyDeviceToDevice, s));
    QMC_CUDA(cudaMemcpyAsync(ar + a.w0_pad + (size_t)o2 * d1, ar + a.w_main[0] + (size_t)kx * d1,
                             sizeof(float) * k2 * d1, cudaMemcpyDeviceToDevice, s));
    QMC_CUDA(launch_transpose_split(s, ar + a.w0_pad, a.k0w, d1, d1, m->arena_bf16 + a.t0_pad, a.k0w, d1));
  }
  for (int l = 0; l < d.L; ++l)
    if (d.upd2[l] && d.d2[l] == 32 && d.d2_in[l] <= 32)
      QMC_CUDA(launch_pair_frags(s, ar + a.w2[l], d.d2_in[l], reinterpret_cast<uint4*>(m->arena_bf16 + a.pfrag[l])));
  m->params_set = true;
  return QMC_OK;
}

size_t qmc_workspace_size(const qmc_model* m, int op, int batch) {
  if (!m || batch < 1) return 0;
  if (m->kind == QMC_KIND_PSIFORMER) {
    if (op == QMC_OP_LOCAL_ENERGY) return psi_fl_check(m) == QMC_OK ? psi_fl_plan(m, psi_fl_chunk(m, batch)).base.total : 0;
    if (op == QMC_OP_GRAD) return psi_grad_workspace(m, batch);
    return op == QMC_OP_FORWARD || op == QMC_OP_MH ? psi_make_plan(m, batch).base.total : 0;
  }
  if (op == QMC_OP_GRAD) return grad_workspace(m, batch);
  return make_plan(m, op, batch).total;
}

qmc_status qmc_model_set_energy_budget(qmc_model* m, size_t bytes) {
  if (!m || bytes == 0) { set_error("null model or zero budget"); return QMC_ERR_ARG; }
  m->energy_budget = bytes;
  return QMC_OK;
}

qmc_status qmc_model_set_det_guard(qmc_model* m, int mode) {
  if (!m || mode < -1 || mode > 1) { set_error("null model or mode outside -1..1"); return QMC_ERR_ARG; }
  m->det_guard = mode;
  return QMC_OK;
}

qmc_status qmc_model_set_grad_budget(qmc_model* m, size_t bytes) {
  if (!m || bytes == 0) { set_error("null model or zero budget"); return QMC_ERR_ARG; }
  m->grad_budget = bytes;
  return QMC_OK;
}

qmc_status qmc_grad(qmc_model* m, int batch, const float* electrons, const double* weights, float* per_walker,
                    double* grad, float* logpsi, void* ws, size_t ws_bytes, cudaStream_t s) {
  if (!m) { set_error("null model"); return QMC_ERR_ARG; }
  if (!m->params_set) { set_error("parameters not set (qmc_model_set_params)"); return QMC_ERR_ARG; }
  if (batch < 1 || !electrons) { set_error("bad batch/electrons"); return QMC_ERR_ARG; }
  if (!per_walker && !grad) { set_error("nothing to compute: per_walker and grad are both null"); return QMC_ERR_ARG; }
  if (grad && !weights) { set_error("grad needs per-walker weights"); return QMC_ERR_ARG; }
  if (!ws) { set_error("null workspace"); return QMC_ERR_WORKSPACE; }
  int dev;
  QMC_CUDA(cudaGetDevice(&dev));
  if (dev != m->device) {
    set_error("model lives on device %d but device %d is current", m->device, dev);
    return QMC_ERR_ARG;
  }
  if (m->kind == QMC_KIND_PSIFORMER)
    return run_psi_grad(m, batch, electrons, weights, per_walker, grad, logpsi, ws, ws_bytes, s);
  return run_grad(m, batch, electrons, weights, per_walker, grad, logpsi, ws, ws_bytes, s);
}

int qmc_layer_taps(const qmc_model* m, int batch, qmc_layer_tap* taps, int max_taps, size_t* total_floats) {
  if (!m || batch < 1 || (max_taps > 0 && !taps)) return -1;
  if (m->kind == QMC_KIND_PSIFORMER) return attn_layer_taps(m, batch, taps, max_taps, total_floats);
  return layer_taps(m, batch, taps, max_taps, total_floats);
}

qmc_status qmc_grad_taps(qmc_model* m, int batch, const float* electrons, float* taps, size_t taps_floats,
                         float* logpsi, void* ws, size_t ws_bytes, cudaStream_t s) {
  if (!m) { set_error("null model"); return QMC_ERR_ARG; }
  if (!m->params_set) { set_error("parameters not set (qmc_model_set_params)"); return QMC_ERR_ARG; }
  if (batch < 1 || !electrons || !taps) { set_error("bad batch/electrons/taps"); return QMC_ERR_ARG; }
  if (!ws) { set_error("null workspace"); return QMC_ERR_WORKSPACE; }
  int dev;
  QMC_CUDA(cudaGetDevice(&dev));
  if (dev != m->device) {
    set_error("model lives on device %d but device %d is current", m->device, dev);
    return QMC_ERR_ARG;
  }
  if (m->kind == QMC_KIND_PSIFORMER)
    return run_attn_grad_taps(m, batch, electrons, taps, taps_floats, logpsi, ws, ws_bytes, s);
  return run_grad_taps(m, batch, electrons, taps, taps_floats, logpsi, ws, ws_bytes, s);
}

qmc_status qmc_forward(qmc_model* m, int batch, const float* electrons, float* logpsi, float* sign,
                       uint8_t* flags, void* ws, size_t ws_bytes, cudaStream_t s) {
  QMC_TRY(check_call(m, batch, ws, ws_bytes, QMC_OP_FORWARD));
  if (!electrons || !logpsi) { set_error("null electrons/logpsi"); return QMC_ERR_ARG; }
  if (m->kind == QMC_KIND_PSIFORMER) return psi_evaluate(m, psi_make_plan(m, batch), ws, electrons, logpsi, sign, flags, s);
  Plan p = make_plan(m, QMC_OP_FORWARD, batch);
  return evaluate(m, p, ws, electrons, false, logpsi, sign, nullptr, nullptr, flags, s);
}

qmc_status qmc_local_energy(qmc_model* m, int batch, const float* electrons, float* e_local, float* ke,
                            float* pe, float* logpsi, uint8_t* flags, void* ws, size_t ws_bytes,
                            cudaStream_t s) {
  QMC_TRY(check_call(m, batch, ws, ws_bytes, QMC_OP_LOCAL_ENERGY));
  if (!electrons || !e_local) { set_error("null electrons/e_local"); return QMC_ERR_ARG; }
  if (m->kind == QMC_KIND_PSIFORMER) return psi_local_energy(m, batch, electrons, e_local, ke, pe, logpsi, flags, ws, s);
  Plan p = make_plan(m, QMC_OP_LOCAL_ENERGY, batch);
  QMC_TRY(evaluate(m, p, ws, electrons, true, logpsi ? logpsi : at<float>(ws, p.lpsi),
                   at<float>(ws, p.sgn), ke, e_local, flags, s));
  if (pe) QMC_CUDA(cudaMemcpyAsync(pe, at<float>(ws, p.pe), sizeof(float) * batch, cudaMemcpyDeviceToDevice, s));
  return QMC_OK;
}

int qmc_tangent_rows(const qmc_model* m, int op) {
  if (!m || op < QMC_OP_FORWARD || op > QMC_OP_GRAD) return -1;
  if (m->kind == QMC_KIND_PSIFORMER) {
    if (op == QMC_OP_LOCAL_ENERGY) return psi_fl_plan(m, 1).base.Tp;
    return op == QMC_OP_FORWARD || op == QMC_OP_MH ? 1 : -1;
  }
  return make_plan(m, op, 1).Tp;
}

qmc_status qmc_mh_steps(qmc_model* m, int batch, int steps, float stddev, uint64_t seed, uint64_t counter,
                        float* electrons, float* log_prob, uint32_t* accepts, const float* inj_normals,
                        const float* inj_uniforms, uint8_t* flags, void* ws, size_t ws_bytes,
                        cudaStream_t s) {
  return qmc::mh_steps(m, batch, steps, stddev, seed, counter, nullptr, electrons, log_prob, accepts,
                       inj_normals, inj_uniforms, flags, ws, ws_bytes, s);
}

qmc_status qmc_mh_steps_resident(qmc_model* m, int batch, int steps, float stddev, uint64_t seed,
                                 uint64_t* counter, float* electrons, float* log_prob, uint32_t* accepts,
                                 uint8_t* flags, void* ws, size_t ws_bytes, cudaStream_t s) {
  if (!counter) { set_error("null device counter"); return QMC_ERR_ARG; }
  QMC_TRY(qmc::mh_steps(m, batch, steps, stddev, seed, 0, counter, electrons, log_prob, accepts, nullptr,
                        nullptr, flags, ws, ws_bytes, s));
  QMC_PROF(QMC_KC_OTHER, launch_counter_add(s, counter, (uint64_t)steps));
  return QMC_OK;
}

qmc_status qmc_mh_steps_grouped(qmc_model* m, int n_jobs, const int* offsets, const uint64_t* seeds,
                                uint64_t* counters, int batch, int steps, float stddev, float* electrons,
                                float* log_prob, uint32_t* accepts, uint8_t* flags, void* ws, size_t ws_bytes,
                                cudaStream_t s) {
  if (n_jobs < 1 || n_jobs > 4096 || !offsets || !seeds || !counters) {
    set_error("grouped MH: 1..4096 jobs and device offsets / seeds / counters");
    return QMC_ERR_ARG;
  }
  MhGroup g;
  g.n_jobs = n_jobs;
  g.offsets = offsets;
  g.seeds = seeds;
  g.counters = counters;
  QMC_TRY(qmc::mh_steps(m, batch, steps, stddev, 0, 0, nullptr, electrons, log_prob, accepts, nullptr, nullptr,
                        flags, ws, ws_bytes, s, g));
  QMC_PROF(QMC_KC_OTHER, launch_counter_add(s, counters, (uint64_t)steps, n_jobs));
  return QMC_OK;
}

qmc_status qmc_mh_draws(const qmc_model* m, int batch, int steps, uint64_t seed, uint64_t counter,
                        float* normals, float* uniforms, cudaStream_t s) {
  if (!m || batch < 1 || steps < 1) { set_error("bad arguments"); return QMC_ERR_ARG; }
  QMC_PROF(QMC_KC_OTHER, launch_mh_draws(s, batch, m->d.n, steps, seed, counter, normals, uniforms));
  return QMC_OK;
}

qmc_status qmc_reduce_mean_var(int batch, const float* x, double* mean_var, cudaStream_t s) {
  if (batch < 1 || !x || !mean_var) { set_error("bad arguments"); return QMC_ERR_ARG; }
  QMC_PROF(QMC_KC_OTHER, launch_reduce_mean_var(s, batch, x, mean_var));
  return QMC_OK;
}

qmc_status qmc_reduce_mean_var_segments(int n_segments, const int* offsets, const float* x, double* mean_var,
                                        cudaStream_t s) {
  if (n_segments < 1 || n_segments > 65535 || !offsets || !x || !mean_var) {
    set_error("bad arguments");
    return QMC_ERR_ARG;
  }
  QMC_PROF(QMC_KC_OTHER, launch_reduce_mean_var(s, 0, x, mean_var, offsets, n_segments));
  return QMC_OK;
}

}  // extern "C"
