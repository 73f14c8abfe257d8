// cpu_fp32.cpp -- FP32 CPU restatement of the NeuralODE gradient evaluation,
// multithreaded over the batch. TEST INFRASTRUCTURE AND CPU BASELINE ONLY: the
// product never links or calls it. It is the timed CPU arm of the benchmark
// (the reference itself is Julia and does not run on these machines) and is
// checked against the FP64 oracle (oracle/tsit5.py) by the CPU test-suite.
//
// What it restates (the same algorithm as oracle/tsit5.py, in FP32 state
// arithmetic with FP64 time, step size and controller):
//  * NeuralODE forward, solve(ODEProblem{false}(dudt, x, tspan, p), Tsit5();
//    saveat, abstol, reltol) at src/neural_de.jl:52-58: Tsit5 with one step
//    size and one RMS error norm over the whole S x B state, the PI
//    controller, the initial-step algorithm, the free interpolant at saveat;
//  * the MLP right-hand side dudt(u, p, t) = model(u, p) (src/neural_de.jl:50),
//    Chain([x -> x.^3,] Dense(d0, d1, act), ...) with tanh / softplus /
//    identity, optionally with t appended as an input row;
//  * the InterpolatingAdjoint gradient (default sensealg, src/neural_de.jl:57):
//    reverse-time Tsit5 on lam with the same controller and tolerances (lam in
//    the error norm, the parameter quadrature mu not), u(t) from the forward's
//    dense output, save points as stops where lam jumps by dL/du(t_i) and the
//    FSAL stage is evaluated again;
//  * the MSE (or SSE) loss at the save points.
//
// Layout: the batch is cut into tiles of kTB trajectories; a state vector is
// [tile][component][kTB] with components padded to a multiple of 4 (padding
// rows stay zero), so that every GEMM streams kTB contiguous floats per
// feature. Each accepted step is independent per trajectory given its step
// size, so one parallel loop over tiles runs all six stages of an attempt and
// only the error norm is reduced across threads. The parameter quadrature is
// accumulated per thread (static schedule: a thread always owns the same
// tiles) and summed over threads in FP64 at the end.
//
// Portable C++ (GCC vector extensions, no intrinsics): builds and gives the
// same results on x86-64 and aarch64.
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>

namespace {

typedef float v4f __attribute__((vector_size(16)));

constexpr int kTB = 64;  // trajectories per tile

// ---- Tsit5 tableau (Tsitouras 2011), FSAL; btilde = b - bhat ----------------------
const double kC[7] = {0.0, 0.161, 0.327, 0.9, 0.9800255409045097, 1.0, 1.0};
const double kA[7][7] = {
    {0, 0, 0, 0, 0, 0, 0},
    {0.161, 0, 0, 0, 0, 0, 0},
    {-0.008480655492356989, 0.335480655492357, 0, 0, 0, 0, 0},
    {2.897153057105493, -6.359448489975075, 4.3622954328695815, 0, 0, 0, 0},
    {5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525, 0, 0, 0},
    {5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383, 0, 0},
    {0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081, 2.324710524099774,
     0}};
const double kBt[7] = {-0.00178001105222577714, -0.0008164344596567469, 0.007880878010261995,
                       -0.1447110071732629,     0.5823571654525552,     -0.45808210592918697,
                       1.0 / 66.0};
// free 4th-order interpolant: b_i(theta) = sum_m R[i][m] theta^(m+1)
const double kR[7][4] = {{1.0, -2.763706197274826, 2.9132554618219126, -1.0530884977290216},
                         {0.0, 0.13169999999999998, -0.2234, 0.1017},
                         {0.0, 3.9302962368947516, -5.941033872131505, 2.490627285651253},
                         {0.0, -12.411077166933676, 30.33818863028232, -16.548102889244902},
                         {0.0, 37.50931341651104, -88.1789048947664, 47.37952196281928},
                         {0.0, -27.896526289197286, 65.09189467479366, -34.87065786149661},
                         {0.0, 1.5, -4.0, 2.5}};
// PI controller (defaults for a 5th-order explicit method)
constexpr double kBeta1 = 7.0 / 50.0, kBeta2 = 2.0 / 25.0, kQmin = 1.0 / 5.0, kQmax = 10.0, kGamma = 9.0 / 10.0,
                 kQoldInit = 1e-4;

enum { RET_SUCCESS = 0, RET_MAXITERS = 1, RET_DTMIN = 2, RET_UNSTABLE = 3 };
enum { ACT_IDENTITY = 0, ACT_TANH = 1, ACT_SOFTPLUS = 2 };

void interp_weights(double th, double* bw) {
  const double pw[4] = {th, th * th, th * th * th, th * th * th * th};
  for (int i = 0; i < 7; ++i) bw[i] = kR[i][0] * pw[0] + kR[i][1] * pw[1] + kR[i][2] * pw[2] + kR[i][3] * pw[3];
}

double pi_q(double eest, double qold, double* q11) {
  if (eest == 0.0) {
    *q11 = 0.0;
    return 1.0 / kQmax;
  }
  const double a = std::pow(eest, kBeta1);
  *q11 = a;
  double q = a / std::pow(qold, kBeta2);
  return std::max(1.0 / kQmax, std::min(1.0 / kQmin, q / kGamma));
}

inline int up4(int n) { return (n + 3) & ~3; }

// ---- the network -------------------------------------------------------------------
struct Net {
  int L = 0, S = 0, Sp = 0;
  bool cube = false, timein = false;
  int d[9] = {}, dp[9] = {}, act[8] = {};
  std::vector<float> WT[8];  // [dp[l]][dp[l+1]]: WT[i][o] = W[o][i] (the flat layout, padded)
  std::vector<float> W[8];   // [dp[l+1]][dp[l]]: W[o][i]
  std::vector<float> b[8];   // [dp[l+1]]
  size_t woff[8] = {}, boff[8] = {}, P = 0;
  size_t gsz = 0;            // floats of a padded gradient buffer
  size_t goff[8] = {}, gboff[8] = {};
  int maxdp = 0;
};

void net_init(Net& n, int L, const int* dims, const int* acts, int cube, int timein, const float* p) {
  n.L = L;
  n.cube = cube != 0;
  n.timein = timein != 0;
  for (int l = 0; l <= L; ++l) {
    n.d[l] = dims[l];
    n.dp[l] = up4(dims[l]);
    n.maxdp = std::max(n.maxdp, n.dp[l]);
  }
  n.S = dims[L];
  n.Sp = up4(n.S);
  size_t o = 0, g = 0;
  for (int l = 0; l < L; ++l) {
    const int in = n.d[l], out = n.d[l + 1], ip = n.dp[l], op = n.dp[l + 1];
    n.act[l] = acts[l];
    n.woff[l] = o;
    n.WT[l].assign((size_t)ip * op, 0.f);
    n.W[l].assign((size_t)op * ip, 0.f);
    for (int i = 0; i < in; ++i)
      for (int k = 0; k < out; ++k) {
        const float w = p[o + (size_t)i * out + k];  // out x in, column-major
        n.WT[l][(size_t)i * op + k] = w;
        n.W[l][(size_t)k * ip + i] = w;
      }
    o += (size_t)in * out;
    n.boff[l] = o;
    n.b[l].assign(op, 0.f);
    for (int k = 0; k < out; ++k) n.b[l][k] = p[o + k];
    o += out;
    n.goff[l] = g;
    g += (size_t)ip * op;
    n.gboff[l] = g;
    g += op;
  }
  n.P = o;
  n.gsz = g;
}

// Y[n][:] = bias[n] + sum_k M[k][n] X[k][:]   (M: K x N row-major, N % 4 == 0;
// X: K x kTB; Y: N x kTB). 4 outputs x 16 trajectories per register block.
void gemm_tile(const float* __restrict__ M, const float* __restrict__ X, float* __restrict__ Y, int K, int N,
               const float* bias) {
  for (int n0 = 0; n0 < N; n0 += 4) {
    for (int b0 = 0; b0 < kTB; b0 += 16) {
      v4f acc[4][4];
      for (int r = 0; r < 4; ++r) {
        const float bv = bias ? bias[n0 + r] : 0.f;
        for (int v = 0; v < 4; ++v) acc[r][v] = (v4f){bv, bv, bv, bv};
      }
      const float* mp = M + n0;
      const float* xp = X + b0;
      for (int k = 0; k < K; ++k) {
        v4f w;
        std::memcpy(&w, mp + (size_t)k * N, sizeof w);
        const v4f* x = reinterpret_cast<const v4f*>(xp + (size_t)k * kTB);
        const v4f x0 = x[0], x1 = x[1], x2 = x[2], x3 = x[3];
        for (int r = 0; r < 4; ++r) {
          const float s = w[r];
          acc[r][0] += s * x0;
          acc[r][1] += s * x1;
          acc[r][2] += s * x2;
          acc[r][3] += s * x3;
        }
      }
      for (int r = 0; r < 4; ++r) {
        v4f* y = reinterpret_cast<v4f*>(Y + (size_t)(n0 + r) * kTB + b0);
        for (int v = 0; v < 4; ++v) y[v] = acc[r][v];
      }
    }
  }
}

// G[i][o] += c * sum_b D[o][b] A[i][b]   (D: Np x kTB, A: Kp x kTB, G: Kp x Np)
void wgrad_tile(const float* __restrict__ D, const float* __restrict__ A, float* __restrict__ G, int Kp, int Np,
                float c) {
  for (int i0 = 0; i0 < Kp; i0 += 4) {
    for (int o0 = 0; o0 < Np; o0 += 4) {
      v4f acc[4][4];
      for (int r = 0; r < 4; ++r)
        for (int s = 0; s < 4; ++s) acc[r][s] = (v4f){0.f, 0.f, 0.f, 0.f};
      for (int b = 0; b < kTB; b += 4) {
        v4f a[4], d[4];
        for (int r = 0; r < 4; ++r) a[r] = *reinterpret_cast<const v4f*>(A + (size_t)(i0 + r) * kTB + b);
        for (int s = 0; s < 4; ++s) d[s] = *reinterpret_cast<const v4f*>(D + (size_t)(o0 + s) * kTB + b);
        for (int r = 0; r < 4; ++r)
          for (int s = 0; s < 4; ++s) acc[r][s] += a[r] * d[s];
      }
      for (int r = 0; r < 4; ++r)
        for (int s = 0; s < 4; ++s) {
          const v4f q = acc[r][s];
          G[(size_t)(i0 + r) * Np + o0 + s] += c * ((q[0] + q[1]) + (q[2] + q[3]));
        }
    }
  }
}

inline float act_f(float z, int a) {
  if (a == ACT_TANH) return std::tanh(z);
  if (a == ACT_SOFTPLUS) return std::max(z, 0.f) + std::log1p(std::exp(-std::fabs(z)));
  return z;
}
// act'(z) from the output y
inline float dact_y(float y, int a) {
  if (a == ACT_TANH) return 1.f - y * y;
  if (a == ACT_SOFTPLUS) return -std::expm1(-y);
  return 1.f;
}

// Per-thread scratch: activations of every layer, two work tiles.
struct Work {
  std::vector<float> a[9];
  std::vector<float> g0, g1, y;
  void init(const Net& n) {
    for (int l = 0; l <= n.L; ++l) a[l].assign((size_t)n.dp[l] * kTB, 0.f);
    g0.assign((size_t)n.maxdp * kTB, 0.f);
    g1.assign((size_t)n.maxdp * kTB, 0.f);
    y.assign((size_t)n.Sp * kTB, 0.f);
  }
};

// Network input a_0 from the state tile U (Sp x kTB): cube prefix, time row.
void net_input(const Net& n, double t, const float* U, Work& w) {
  float* a0 = w.a[0].data();
  const int S = n.S;
  for (int s = 0; s < S; ++s)
    for (int b = 0; b < kTB; ++b) {
      const float u = U[(size_t)s * kTB + b];
      a0[(size_t)s * kTB + b] = n.cube ? u * u * u : u;
    }
  if (n.timein)
    for (int b = 0; b < kTB; ++b) a0[(size_t)S * kTB + b] = (float)t;
}

// Forward through the layers from a_0; activations kept in w.a[1..L].
void net_forward(const Net& n, Work& w) {
  for (int l = 0; l < n.L; ++l) {
    const int op = n.dp[l + 1], out = n.d[l + 1];
    float* z = w.a[l + 1].data();
    gemm_tile(n.WT[l].data(), w.a[l].data(), z, n.dp[l], op, n.b[l].data());
    const int a = n.act[l];
    if (a != ACT_IDENTITY)
      for (size_t i = 0; i < (size_t)out * kTB; ++i) z[i] = act_f(z[i], a);
    // padding rows stay zero (softplus(0) != 0)
    std::memset(z + (size_t)out * kTB, 0, (size_t)(op - out) * kTB * sizeof(float));
  }
}

// k = f(U, t)
void rhs_tile(const Net& n, double t, const float* U, float* K, Work& w) {
  net_input(n, t, U, w);
  net_forward(n, w);
  std::memcpy(K, w.a[n.L].data(), (size_t)n.Sp * kTB * sizeof(float));
}

// GU = (df/du)^T LAM on the tile and G += c (df/dp)^T LAM summed over the
// tile's valid trajectories (LAM is zero on the others).
void vjp_tile(const Net& n, double t, const float* U, const float* LAM, float* GU, float* G, float c, Work& w) {
  net_input(n, t, U, w);
  net_forward(n, w);
  float* g = w.g0.data();
  float* gn = w.g1.data();
  std::memcpy(g, LAM, (size_t)n.Sp * kTB * sizeof(float));
  for (int l = n.L - 1; l >= 0; --l) {
    const int op = n.dp[l + 1], out = n.d[l + 1], ip = n.dp[l];
    const float* y = w.a[l + 1].data();
    const int a = n.act[l];
    if (a != ACT_IDENTITY)
      for (size_t i = 0; i < (size_t)out * kTB; ++i) g[i] *= dact_y(y[i], a);
    if (G) {
      wgrad_tile(g, w.a[l].data(), G + n.goff[l], ip, op, c);
      float* gb = G + n.gboff[l];
      for (int o = 0; o < out; ++o) {
        float s = 0.f;
        for (int b = 0; b < kTB; ++b) s += g[(size_t)o * kTB + b];
        gb[o] += c * s;
      }
    }
    gemm_tile(n.W[l].data(), g, gn, op, ip, nullptr);
    std::swap(g, gn);
  }
  // g: dL/d(a_0); the state part, through the cube prefix
  for (int s = 0; s < n.S; ++s)
    for (int b = 0; b < kTB; ++b) {
      float v = g[(size_t)s * kTB + b];
      if (n.cube) {
        const float u = U[(size_t)s * kTB + b];
        v *= 3.f * u * u;
      }
      GU[(size_t)s * kTB + b] = v;
    }
  std::memset(GU + (size_t)n.S * kTB, 0, (size_t)(n.Sp - n.S) * kTB * sizeof(float));
}

// ---- solver ---------------------------------------------------------------------------
// A dense-output slot of one accepted forward step: t_n, h_n and the 8
// tile-layout vectors (u_n, k1..k7).
struct Slot {
  double t = 0, h = 0;
  std::unique_ptr<float[]> v;
};

struct Ctx {
  Net net;
  int S = 0, B = 0, ntiles = 0, nthreads = 1;
  size_t tvs = 0;  // floats per tile of one state vector (Sp x kTB)
  size_t nv = 0;   // floats of one state vector (ntiles x tvs)
  std::vector<Work> work;                 // per thread
  std::vector<std::vector<float>> g1, gm, g7;  // per thread: pending quadrature (P1, P_mid, P7)
  std::vector<std::vector<double>> mu;    // per thread: committed quadrature
  std::vector<std::unique_ptr<float[]>> pool;  // reusable 8-vector slots
  std::vector<Slot> slots;                // accepted forward steps of the last solve
  std::vector<float> lam[2], kl[7], ynew, tmp;
  std::vector<double> part;               // per-tile partial sums (fixed summation order)
  long long nf = 0, nacc = 0, nrej = 0, nf_adj = 0, nacc_adj = 0, nrej_adj = 0;
  int ret = RET_SUCCESS, ret_adj = RET_SUCCESS;

  float* tile(std::vector<float>& v, int t) { return v.data() + (size_t)t * tvs; }
  float* tile(float* v, int t) { return v + (size_t)t * tvs; }
  std::unique_ptr<float[]> get_slot() {
    if (!pool.empty()) {
      auto p = std::move(pool.back());
      pool.pop_back();
      return p;
    }
    return std::unique_ptr<float[]>(new float[8 * nv]);
  }
  void recycle() {
    for (auto& s : slots) pool.push_back(std::move(s.v));
    slots.clear();
  }
  double sum_parts() const {
    double s = 0.0;
    for (double x : part) s += x;
    return s;
  }
};

inline bool valid(const Ctx& c, int t, int b) { return t * kTB + b < c.B; }

// The S state rows of the valid trajectories of one tile: sum of f(index).
template <class F>
double tile_sum(const Ctx& c, int t, F f) {
  double s = 0.0;
  for (int r = 0; r < c.S; ++r)
    for (int b = 0; b < kTB; ++b)
      if (valid(c, t, b)) s += f((size_t)r * kTB + b);
  return s;
}

// column-major S x B <-> tile layout
void to_tiles(const Ctx& c, const float* cm, float* tl) {
#pragma omp parallel for schedule(static)
  for (int t = 0; t < c.ntiles; ++t) {
    float* d = tl + (size_t)t * c.tvs;
    std::memset(d, 0, c.tvs * sizeof(float));
    for (int b = 0; b < kTB; ++b)
      if (valid(c, t, b))
        for (int r = 0; r < c.S; ++r) d[(size_t)r * kTB + b] = cm[(size_t)(t * kTB + b) * c.S + r];
  }
}
void from_tiles(const Ctx& c, const float* tl, float* cm) {
#pragma omp parallel for schedule(static)
  for (int t = 0; t < c.ntiles; ++t) {
    const float* s = tl + (size_t)t * c.tvs;
    for (int b = 0; b < kTB; ++b)
      if (valid(c, t, b))
        for (int r = 0; r < c.S; ++r) cm[(size_t)(t * kTB + b) * c.S + r] = s[(size_t)r * kTB + b];
  }
}

// u(t) on tile `t` from the forward's dense output: step n, weights hb.
void dense_setup(const Ctx& c, double tq, int* n, float* hb) {
  int lo = 0, hi = (int)c.slots.size() - 1, k = 0;
  while (lo <= hi) {  // last step with t_n <= tq
    const int mid = (lo + hi) / 2;
    if (c.slots[mid].t <= tq) { k = mid; lo = mid + 1; }
    else hi = mid - 1;
  }
  const Slot& s = c.slots[k];
  double bw[7];
  interp_weights((tq - s.t) / s.h, bw);
  for (int j = 0; j < 7; ++j) hb[j] = (float)(s.h * bw[j]);
  *n = k;
}
void dense_u(const Ctx& c, int n, const float* hb, int t, float* out) {
  const float* v = c.slots[n].v.get() + (size_t)t * c.tvs;
  const size_t m = c.tvs;
  for (size_t i = 0; i < m; ++i) {
    float e = 0.f;
    for (int j = 0; j < 7; ++j) e += hb[j] * v[(size_t)(j + 1) * c.nv + i];
    out[i] = v[i] + e;
  }
}

// Forward solve from u0 (column-major) with saves into usave (S x B x nsave).
void forward(Ctx& c, const float* u0, double t0, double t1, const double* saveat, int nsave, double abstol,
             double reltol, long long maxiters, float* usave) {
  c.recycle();
  c.nf = c.nacc = c.nrej = 0;
  c.ret = RET_SUCCESS;
  const double N = (double)c.S * c.B, dtmax = std::fabs(t1 - t0);
  auto cur = c.get_slot();
  float* u = cur.get();
  to_tiles(c, u0, u);
  float* kv[7];
  auto setk = [&](float* base) {
    for (int j = 0; j < 7; ++j) kv[j] = base + (size_t)(j + 1) * c.nv;
  };
  setk(cur.get());
#pragma omp parallel for schedule(static)
  for (int t = 0; t < c.ntiles; ++t) rhs_tile(c.net, t0, c.tile(u, t), c.tile(kv[0], t), c.work[omp_get_thread_num()]);
  c.nf = 1;
  const size_t SB = (size_t)c.S * c.B;
  int isave = 0;
  while (isave < nsave && saveat[isave] == t0) {
    std::memcpy(usave + (size_t)isave * SB, u0, SB * sizeof(float));
    ++isave;
  }
  // initial step (Hairer's algorithm as the integrator implements it)
  double dt;
  {
#pragma omp parallel for schedule(static)
    for (int t = 0; t < c.ntiles; ++t) {
      const float* ut = c.tile(u, t);
      const float* ft = c.tile(kv[0], t);
      double s0 = 0, s1 = 0;
      tile_sum(c, t, [&](size_t i) {
        const double sk = abstol + std::fabs((double)ut[i]) * reltol;
        s0 += ((double)ut[i] / sk) * ((double)ut[i] / sk);
        s1 += ((double)ft[i] / sk) * ((double)ft[i] / sk);
        return 0.0;
      });
      c.part[2 * t] = s0;
      c.part[2 * t + 1] = s1;
    }
    double s0 = 0, s1 = 0;
    for (int t = 0; t < c.ntiles; ++t) { s0 += c.part[2 * t]; s1 += c.part[2 * t + 1]; }
    const double d0 = std::sqrt(s0 / N), d1 = std::sqrt(s1 / N);
    double dt0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * (d0 / d1);
    dt0 = std::min(dt0, dtmax);
    const float hf = (float)dt0;
#pragma omp parallel for schedule(static)
    for (int t = 0; t < c.ntiles; ++t) {
      Work& w = c.work[omp_get_thread_num()];
      const float* ut = c.tile(u, t);
      const float* f0 = c.tile(kv[0], t);
      float* y = w.y.data();
      for (size_t i = 0; i < c.tvs; ++i) y[i] = ut[i] + hf * f0[i];
      float* f1 = c.tile(c.tmp, t);
      rhs_tile(c.net, t0 + dt0, y, f1, w);
      c.part[2 * t] = tile_sum(c, t, [&](size_t i) {
        const double sk = abstol + std::fabs((double)ut[i]) * reltol;
        const double z = ((double)f1[i] - (double)f0[i]) / sk;
        return z * z;
      });
    }
    double s2 = 0;
    for (int t = 0; t < c.ntiles; ++t) s2 += c.part[2 * t];
    c.nf += 1;
    const double d2 = std::sqrt(s2 / N) / dt0;
    const double m = std::max(d1, d2);
    const double dt1 = (m <= 1e-15) ? std::max(1e-6, dt0 * 1e-3) : std::pow(10.0, -(2.0 + std::log10(m)) / 5.0);
    dt = std::min(100.0 * dt0, std::min(dt1, dtmax));
  }
  double t = t0, qold = kQoldInit;
  long long iter = 0;
  while (t1 - t > 0.0) {
    if (iter >= maxiters) { c.ret = RET_MAXITERS; break; }
    ++iter;
    const double rem = t1 - t;
    const bool clipped = dt >= rem;
    const double h = clipped ? rem : dt;
    float ha[7][7], hbt[7];
    for (int i = 0; i < 7; ++i)
      for (int j = 0; j < 7; ++j) ha[i][j] = (float)(h * kA[i][j]);
    for (int j = 0; j < 7; ++j) hbt[j] = (float)(h * kBt[j]);
    float* yn = c.ynew.data();
#pragma omp parallel for schedule(static)
    for (int tt = 0; tt < c.ntiles; ++tt) {
      Work& w = c.work[omp_get_thread_num()];
      const float* ut = c.tile(u, tt);
      float* y = w.y.data();
      for (int i = 1; i < 7; ++i) {
        for (size_t q = 0; q < c.tvs; ++q) {
          float s = 0.f;
          for (int j = 0; j < i; ++j) s += ha[i][j] * kv[j][(size_t)tt * c.tvs + q];
          y[q] = ut[q] + s;
        }
        rhs_tile(c.net, t + kC[i] * h, y, c.tile(kv[i], tt), w);
      }
      float* ynt = c.tile(yn, tt);
      std::memcpy(ynt, y, c.tvs * sizeof(float));
      c.part[tt] = tile_sum(c, tt, [&](size_t q) {
        float e = 0.f;
        for (int j = 0; j < 7; ++j) e += hbt[j] * kv[j][(size_t)tt * c.tvs + q];
        const double sc = abstol + std::max(std::fabs((double)ut[q]), std::fabs((double)ynt[q])) * reltol;
        const double r = (double)e / sc;
        return std::isfinite(ynt[q]) ? r * r : (double)INFINITY;
      });
    }
    c.nf += 6;
    double se = 0;
    for (int tt = 0; tt < c.ntiles; ++tt) se += c.part[tt];
    const double eest = std::sqrt(se / N);
    if (!std::isfinite(eest)) { c.ret = RET_UNSTABLE; break; }
    double q11;
    double q = pi_q(eest, qold, &q11);
    if (eest <= 1.0) {
      const double tnew = clipped ? t1 : t + h;
      while (isave < nsave && saveat[isave] - tnew <= 0.0) {
        const double sv = saveat[isave];
        std::vector<float>& o = c.tmp;
        if (sv == tnew) {
          from_tiles(c, yn, usave + (size_t)isave * SB);
        } else {
          double bw[7];
          interp_weights((sv - t) / h, bw);
          float hb[7];
          for (int j = 0; j < 7; ++j) hb[j] = (float)(h * bw[j]);
#pragma omp parallel for schedule(static)
          for (int tt = 0; tt < c.ntiles; ++tt)
            for (size_t qq = 0; qq < c.tvs; ++qq) {
              const size_t i = (size_t)tt * c.tvs + qq;
              float e = 0.f;
              for (int j = 0; j < 7; ++j) e += hb[j] * kv[j][i];
              o[i] = u[i] + e;
            }
          from_tiles(c, o.data(), usave + (size_t)isave * SB);
        }
        ++isave;
      }
      Slot sl;
      sl.t = t;
      sl.h = h;
      sl.v = std::move(cur);
      c.slots.push_back(std::move(sl));
      cur = c.get_slot();
      u = cur.get();
      std::memcpy(u, yn, c.nv * sizeof(float));
      std::memcpy(cur.get() + c.nv, kv[6], c.nv * sizeof(float));  // FSAL
      setk(cur.get());
      ++c.nacc;
      t = tnew;
      if (q >= 1.0 && q <= 1.0) q = 1.0;
      qold = std::max(eest, kQoldInit);
      dt = std::min(h / q, dtmax);
    } else {
      ++c.nrej;
      dt = h / std::min(1.0 / kQmin, q11 / kGamma);
    }
  }
  c.pool.push_back(std::move(cur));
}

// InterpolatingAdjoint from the cotangent dLdu (S x B x nsave) of the saves;
// dLdu0: S x B, dLdp: flat parameters.
void adjoint(Ctx& c, const double* saveat, int nsave, double t0, double abstol, double reltol,
             long long maxiters, const float* dLdu, float* dLdu0, float* dLdp) {
  const Net& n = c.net;
  const size_t SB = (size_t)c.S * c.B;
  const double N = (double)SB;
  c.nf_adj = c.nacc_adj = c.nrej_adj = 0;
  c.ret_adj = RET_SUCCESS;
  std::vector<double> stops;  // distinct save times, descending
  for (int i = 0; i < nsave; ++i) stops.push_back(saveat[i]);
  std::sort(stops.begin(), stops.end(), [](double a, double b) { return a > b; });
  stops.erase(std::unique(stops.begin(), stops.end()), stops.end());
  const double tlast = stops[0];
  // cotangent jump at time s, added into tile-layout lam
  auto jump = [&](double s, float* lam) {
    std::vector<float>& tl = c.tmp;
    for (int i = 0; i < nsave; ++i)
      if (saveat[i] == s) {
        to_tiles(c, dLdu + (size_t)i * SB, tl.data());
        for (size_t q = 0; q < c.nv; ++q) lam[q] += tl[q];
      }
  };
  float* lam = c.lam[0].data();
  std::memset(lam, 0, c.nv * sizeof(float));
  jump(tlast, lam);
  for (auto& m : c.mu) std::fill(m.begin(), m.end(), 0.0);
  int k1i = 0;  // kl[k1i] holds K1 (the other of kl[0] / kl[6] holds K7)
  auto K = [&](int j) -> float* {
    if (j == 0) return c.kl[k1i].data();
    if (j == 6) return c.kl[6 - k1i].data();
    return c.kl[j].data();
  };
  std::vector<float>* P1 = c.g1.data();
  std::vector<float>* P7 = c.g7.data();
  // K1 = -(df/du)^T lam at (t, u(t)); P1 = (df/dp)^T lam per thread
  auto fsal = [&](double tq) {
    int sn;
    float hb[7];
    dense_setup(c, tq, &sn, hb);
#pragma omp parallel
    {
      const int tid = omp_get_thread_num();
      std::fill(P1[tid].begin(), P1[tid].end(), 0.f);
#pragma omp for schedule(static)
      for (int tt = 0; tt < c.ntiles; ++tt) {
        Work& w = c.work[tid];
        float* ut = w.y.data();
        dense_u(c, sn, hb, tt, ut);
        float* k = c.tile(K(0), tt);
        vjp_tile(n, tq, ut, c.tile(lam, tt), k, P1[tid].data(), 1.f, w);
        for (size_t q = 0; q < c.tvs; ++q) k[q] = -k[q];
      }
    }
    c.nf_adj += 1;
  };
  double t = tlast;
  if (tlast > t0) {
    fsal(t);
    const double dtmax = tlast - t0;
    // initial step
    double dt;
    {
#pragma omp parallel for schedule(static)
      for (int tt = 0; tt < c.ntiles; ++tt) {
        const float* l = c.tile(lam, tt);
        const float* f = c.tile(K(0), tt);
        double s0 = 0, s1 = 0;
        tile_sum(c, tt, [&](size_t i) {
          const double sk = abstol + std::fabs((double)l[i]) * reltol;
          s0 += ((double)l[i] / sk) * ((double)l[i] / sk);
          s1 += ((double)f[i] / sk) * ((double)f[i] / sk);
          return 0.0;
        });
        c.part[2 * tt] = s0;
        c.part[2 * tt + 1] = s1;
      }
      double s0 = 0, s1 = 0;
      for (int tt = 0; tt < c.ntiles; ++tt) { s0 += c.part[2 * tt]; s1 += c.part[2 * tt + 1]; }
      const double d0 = std::sqrt(s0 / N), d1 = std::sqrt(s1 / N);
      double dt0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * (d0 / d1);
      dt0 = std::min(dt0, dtmax);
      const float hf = (float)(-dt0);
      int sn;
      float hb[7];
      dense_setup(c, t - dt0, &sn, hb);
#pragma omp parallel for schedule(static)
      for (int tt = 0; tt < c.ntiles; ++tt) {
        Work& w = c.work[omp_get_thread_num()];
        const float* l = c.tile(lam, tt);
        const float* f0 = c.tile(K(0), tt);
        std::vector<float> ybuf(c.tvs), ub(c.tvs);
        for (size_t i = 0; i < c.tvs; ++i) ybuf[i] = l[i] + hf * f0[i];
        dense_u(c, sn, hb, tt, ub.data());
        float* f1 = c.tile(c.tmp, tt);
        vjp_tile(n, t - dt0, ub.data(), ybuf.data(), f1, nullptr, 0.f, w);
        c.part[2 * tt] = tile_sum(c, tt, [&](size_t i) {
          const double sk = abstol + std::fabs((double)l[i]) * reltol;
          const double z = (-(double)f1[i] - (double)f0[i]) / sk;
          return z * z;
        });
      }
      double s2 = 0;
      for (int tt = 0; tt < c.ntiles; ++tt) s2 += c.part[2 * tt];
      c.nf_adj += 1;
      const double d2 = std::sqrt(s2 / N) / dt0;
      const double m = std::max(d1, d2);
      const double dt1 =
          (m <= 1e-15) ? std::max(1e-6, dt0 * 1e-3) : std::pow(10.0, -(2.0 + std::log10(m)) / 5.0);
      dt = std::min(100.0 * dt0, std::min(dt1, dtmax));
    }
    double qold = kQoldInit;
    long long iter = 0;
    size_t istop = 1;  // next stop: stops[istop] (or t0 past the list)
    float* lnew = c.lam[1].data();
    while (t - t0 > 0.0) {
      if (iter >= maxiters) { c.ret_adj = RET_MAXITERS; break; }
      ++iter;
      const double stop = istop < stops.size() && stops[istop] > t0 ? stops[istop] : t0;
      const double rem = t - stop;
      const bool clipped = dt >= rem;
      const double H = clipped ? rem : dt;
      const double h = -H;
      float ha[7][7], hbt[7];
      for (int i = 0; i < 7; ++i)
        for (int j = 0; j < 7; ++j) ha[i][j] = (float)(h * kA[i][j]);
      for (int j = 0; j < 7; ++j) hbt[j] = (float)(h * kBt[j]);
      int sn[7];
      float shb[7][7];
      for (int i = 1; i < 7; ++i) dense_setup(c, t + kC[i] * h, &sn[i], shb[i]);
      float* ln = lnew;
#pragma omp parallel
      {
        const int tid = omp_get_thread_num();
        Work& w = c.work[tid];
        std::fill(c.gm[tid].begin(), c.gm[tid].end(), 0.f);
        std::fill(P7[tid].begin(), P7[tid].end(), 0.f);
        std::vector<float> ub(c.tvs);
#pragma omp for schedule(static)
        for (int tt = 0; tt < c.ntiles; ++tt) {
          const float* lt = c.tile(lam, tt);
          float* y = w.y.data();
          for (int i = 1; i < 7; ++i) {
            for (size_t q = 0; q < c.tvs; ++q) {
              float s = 0.f;
              for (int j = 0; j < i; ++j) s += ha[i][j] * K(j)[(size_t)tt * c.tvs + q];
              y[q] = lt[q] + s;
            }
            dense_u(c, sn[i], shb[i], tt, ub.data());
            float* k = c.tile(K(i), tt);
            float* G = i < 6 ? c.gm[tid].data() : P7[tid].data();
            vjp_tile(n, t + kC[i] * h, ub.data(), y, k, G, i < 6 ? (float)kA[6][i] : 1.f, w);
            for (size_t q = 0; q < c.tvs; ++q) k[q] = -k[q];
          }
          float* lnt = c.tile(ln, tt);
          std::memcpy(lnt, y, c.tvs * sizeof(float));
          c.part[tt] = tile_sum(c, tt, [&](size_t q) {
            float e = 0.f;
            for (int j = 0; j < 7; ++j) e += hbt[j] * K(j)[(size_t)tt * c.tvs + q];
            const double sc = abstol + std::max(std::fabs((double)lt[q]), std::fabs((double)lnt[q])) * reltol;
            const double r = (double)e / sc;
            return std::isfinite(lnt[q]) ? r * r : (double)INFINITY;
          });
        }
      }
      c.nf_adj += 6;
      double se = 0;
      for (int tt = 0; tt < c.ntiles; ++tt) se += c.part[tt];
      const double eest = std::sqrt(se / N);
      if (!std::isfinite(eest)) { c.ret_adj = RET_UNSTABLE; break; }
      double q11;
      double q = pi_q(eest, qold, &q11);
      if (eest <= 1.0) {
        const double b1 = kA[6][0];
#pragma omp parallel
        {
          const int tid = omp_get_thread_num();
          std::vector<double>& m = c.mu[tid];
          const float* p1 = P1[tid].data();
          const float* pm = c.gm[tid].data();
          for (size_t i = 0; i < n.gsz; ++i) m[i] += H * ((double)b1 * (double)p1[i] + (double)pm[i]);
        }
        std::swap(P1, P7);
        std::swap(lam, lnew);
        k1i = 6 - k1i;  // K7 becomes K1
        ++c.nacc_adj;
        t = clipped ? stop : t + h;
        if (clipped && stop > t0) {
          jump(stop, lam);
          fsal(t);
          ++istop;
        }
        if (q >= 1.0 && q <= 1.0) q = 1.0;
        qold = std::max(eest, kQoldInit);
        dt = std::min(H / q, dtmax);
      } else {
        ++c.nrej_adj;
        dt = H / std::min(1.0 / kQmin, q11 / kGamma);
      }
    }
    if (saveat[0] == t0 || std::find(saveat, saveat + nsave, t0) != saveat + nsave) jump(t0, lam);
  }
  from_tiles(c, lam, dLdu0);
  // dL/dp: sum over threads (FP64), padded layout -> flat layout
  std::vector<double> g(n.gsz, 0.0);
  for (auto& m : c.mu)
    for (size_t i = 0; i < n.gsz; ++i) g[i] += m[i];
  for (int l = 0; l < n.L; ++l) {
    const int in = n.d[l], out = n.d[l + 1], op = n.dp[l + 1];
    for (int i = 0; i < in; ++i)
      for (int k = 0; k < out; ++k) dLdp[n.woff[l] + (size_t)i * out + k] = (float)g[n.goff[l] + (size_t)i * op + k];
    for (int k = 0; k < out; ++k) dLdp[n.boff[l] + k] = (float)g[n.gboff[l] + k];
  }
}

}  // namespace

extern "C" {

// Context for one network (flat parameters p) and batch size.
void* cpuf32_create(int nlayers, const int* dims, const int* acts, int cube, int timein, const float* p, int B,
                    int nthreads) {
  if (nlayers < 1 || nlayers > 8 || B < 1) return nullptr;
  Ctx* c = new Ctx();
  net_init(c->net, nlayers, dims, acts, cube, timein, p);
  c->S = c->net.S;
  c->B = B;
  c->ntiles = (B + kTB - 1) / kTB;
  c->tvs = (size_t)c->net.Sp * kTB;
  c->nv = (size_t)c->ntiles * c->tvs;
  c->nthreads = nthreads > 0 ? nthreads : omp_get_max_threads();
  omp_set_num_threads(c->nthreads);
  c->work.resize(c->nthreads);
  for (auto& w : c->work) w.init(c->net);
  c->g1.assign(c->nthreads, std::vector<float>(c->net.gsz, 0.f));
  c->gm.assign(c->nthreads, std::vector<float>(c->net.gsz, 0.f));
  c->g7.assign(c->nthreads, std::vector<float>(c->net.gsz, 0.f));
  c->mu.assign(c->nthreads, std::vector<double>(c->net.gsz, 0.0));
  c->lam[0].assign(c->nv, 0.f);
  c->lam[1].assign(c->nv, 0.f);
  for (auto& k : c->kl) k.assign(c->nv, 0.f);
  c->ynew.assign(c->nv, 0.f);
  c->tmp.assign(c->nv, 0.f);
  c->part.assign(2 * (size_t)c->ntiles, 0.0);
  return c;
}

void cpuf32_destroy(void* h) { delete static_cast<Ctx*>(h); }

size_t cpuf32_nparams(void* h) { return static_cast<Ctx*>(h)->net.P; }

// One gradient evaluation: forward solve with saves, the loss of the saves
// against target (loss_kind 0: sum of squares, 1: mean of squares), and the
// InterpolatingAdjoint gradient. usave may be NULL. counts[8] receives
// nf, naccept, nreject, nf_adj, naccept_adj, nreject_adj, retcode, retcode_adj.
// Returns 0, or -1 when the forward solve failed (no gradient).
int cpuf32_grad(void* h, const float* u0, double t0, double t1, const double* saveat, int nsave, double abstol,
                double reltol, long long maxiters, const float* target, int loss_kind, double* loss,
                float* usave, float* dLdu0, float* dLdp, long long* counts) {
  Ctx& c = *static_cast<Ctx*>(h);
  omp_set_num_threads(c.nthreads);
  const size_t SB = (size_t)c.S * c.B, n = SB * (size_t)nsave;
  std::vector<float> us(n), dl(n);
  forward(c, u0, t0, t1, saveat, nsave, abstol, reltol, maxiters, us.data());
  counts[0] = c.nf;
  counts[1] = c.nacc;
  counts[2] = c.nrej;
  counts[6] = c.ret;
  counts[3] = counts[4] = counts[5] = counts[7] = 0;
  if (usave) std::memcpy(usave, us.data(), n * sizeof(float));
  if (c.ret != RET_SUCCESS) return -1;
  const double scale = loss_kind == 1 ? 2.0 / (double)n : 2.0;
  double s = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : s)
  for (long long i = 0; i < (long long)n; ++i) {
    const double d = (double)us[i] - (double)target[i];
    s += d * d;
    dl[i] = (float)(scale * d);
  }
  *loss = loss_kind == 1 ? s / (double)n : s;
  adjoint(c, saveat, nsave, t0, abstol, reltol, maxiters, dl.data(), dLdu0, dLdp);
  counts[3] = c.nf_adj;
  counts[4] = c.nacc_adj;
  counts[5] = c.nrej_adj;
  counts[7] = c.ret_adj;
  return 0;
}

}  // extern "C"
