// Initial-condition builders and the quadrature L2 error on the device
// (IGR_adjoints_2d/initial_conditions.jl:15-232, IGR_adjoints_1d/
// initial_conditions.jl:94-204): every node of every instance of a batch in
// one grid-stride launch, so parameter sweeps build their inputs in HBM.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "igr_engine.h"

namespace igrgpu {

namespace {
constexpr double kPi = 3.14159265358979323846;
constexpr int OSEEN_TAB = 4000;  // initial_conditions.jl:187

struct Ic2DArgs {
  const Inst2D* inst; int ninst; BasisDev B;
  int type;
  const double* amps;      // per instance
  double prm[15];
  const double* tables;    // Oseen enthalpy-defect tables, OSEEN_TAB per instance
  double* q[4];
  long long NG;
};

__device__ double oseen_defect_dev(const double* D, double r, double r_max) {
  if (r >= r_max) return 0.0;
  const double t = r / r_max * (OSEEN_TAB - 1) + 1;
  int i = (int)floor(t);
  i = min(max(i, 1), OSEEN_TAB - 1);
  const double w = t - i;
  return (1 - w) * D[i - 1] + w * D[i];
}

__global__ void k2_build_ic(Ic2DArgs a) {
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < a.NG; n += (long long)gridDim.x * blockDim.x) {
    const int ii = find_inst(a.inst, a.ninst, n);
    const Inst2D I = a.inst[ii];
    double c, x, y;
    node_coords2d(a.B, I, n - I.off, &c, &x, &y);
    const double g = I.gamma, A = a.amps[ii];
    const double* prm = a.prm;
    double rho = 1.0, ux = 0.0, uy = 0.0, p = 1.0;
    switch (a.type) {
      case 0: rho = prm[0]; ux = prm[1]; uy = prm[2]; p = prm[3]; break;  // init_constant_state, :15-22
      case 1: {  // init_isentropic_vortex, :39-67 (centre of the domain)
        const double beta = prm[0];
        const double dx = x - I.lx / 2, dy = y - I.ly / 2;
        const double r2 = dx * dx + dy * dy;
        const double ef = exp((1 - r2) / 2);
        const double dT = -(g - 1) * (beta * beta) / (8 * g * (kPi * kPi)) * exp(1 - r2);
        rho = pow(1 + dT, 1 / (g - 1));
        ux = prm[1] - dy * (beta / (2 * kPi)) * ef;
        uy = prm[2] + dx * (beta / (2 * kPi)) * ef;
        p = pow(rho, g);
        break;
      }
      case 2: {  // build_taylor_green_ic!, :105-121
        const double cx = 2 * kPi * x / I.lx, cy = 2 * kPi * y / I.ly;
        ux = A * sin(cx) * cos(cy);
        uy = -A * cos(cx) * sin(cy);
        break;
      }
      case 3: {  // build_sedov_blast_ic!, :136-150
        const double dx = x - I.lx / 2, dy = y - I.ly / 2;
        p = prm[0] + A * exp(-(dx * dx + dy * dy) / (prm[1] * prm[1]));
        break;
      }
      case 4: {  // build_oseen_pair_blast_ic!, :175-231 (velocity over 3 x 3 periodic images)
        const double a_core = prm[0], L = I.lx;
        const double Gam = prm[1] * sqrt(g) * 2 * kPi * a_core / 0.6383;
        const double r_max = 2.0 * L;
        const double* D = a.tables + (long long)ii * OSEEN_TAB;
        double h = g / (g - 1);
        for (int k = 0; k < 2; ++k) {
          const double xc = prm[5 + 3 * k], yc = prm[6 + 3 * k], Gk = prm[7 + 3 * k] * Gam;
          for (int sx = -1; sx <= 1; ++sx)
            for (int sy = -1; sy <= 1; ++sy) {
              const double dx = x - (xc + sx * L), dy = y - (yc + sy * L);
              const double r2 = dx * dx + dy * dy;
              if (r2 < 1e-24) continue;
              const double vr = Gk / (2 * kPi * r2) * (1.0 - exp(-r2 / (a_core * a_core)));
              ux -= vr * dy;
              uy += vr * dx;
            }
          double dx = x - xc, dy = y - yc;
          dx -= L * rint(dx / L);
          dy -= L * rint(dy / L);
          h -= oseen_defect_dev(D, sqrt(dx * dx + dy * dy), r_max);
        }
        const double p_vort = pow((g - 1) * h / g, g / (g - 1));
        rho = pow(p_vort, 1.0 / g);
        const double r2b = (x - prm[2]) * (x - prm[2]) + (y - prm[3]) * (y - prm[3]);
        p = p_vort + A * exp(-r2b / (prm[4] * prm[4]));
        break;
      }
      case 5: {  // several Gaussian blasts (the paper scripts' Sedov state); blast 1's amplitude is A
        const int nb = (int)prm[2];
        double pv = prm[0];
        for (int k = 0; k < nb; ++k) {
          const double dx = x - prm[3 + 3 * k], dy = y - prm[4 + 3 * k];
          pv += (k == 0 ? A : prm[5 + 3 * k]) * exp(-(dx * dx + dy * dy) / (prm[1] * prm[1]));
        }
        p = pv;
        break;
      }
      default: break;
    }
    a.q[2][n] = rho;
    a.q[0][n] = rho * ux;
    a.q[1][n] = rho * uy;
    a.q[3][n] = p / (g - 1) + 0.5 * rho * (ux * ux + uy * uy);
  }
}

struct Ic1DArgs {
  const Inst1D* inst; int ninst; BasisDev B;
  int type;
  const double* amps;
  double* q;  // batch layout: instance i's (mu, rho, E) at 3 off_i
  long long NG;
};

__device__ __forceinline__ int find_inst1(const Inst1D* inst, int ninst, long long n) {
  int lo = 0, hi = ninst - 1;
  while (lo < hi) { const int mid = (lo + hi + 1) / 2; if (inst[mid].off <= n) lo = mid; else hi = mid - 1; }
  return lo;
}

__global__ void k1_build_ic(Ic1DArgs a) {
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < a.NG; n += (long long)gridDim.x * blockDim.x) {
    const int ii = find_inst1(a.inst, a.ninst, n);
    const Inst1D I = a.inst[ii];
    const long long m = n - I.off;
    const int N = a.B.np * I.ne;
    const int e = (int)(m / a.B.np), i = (int)(m % a.B.np);
    const double x = e * I.dx + I.J * (1.0 + a.B.xi[i]);
    const double s = sin(2 * kPi * x / I.L), A = a.amps[ii], g = I.gamma;
    double rho = 1.0, u = 0.0, p = 1.0;
    switch (a.type) {
      case 0: rho = 1 + A * s; u = A * s; p = 1 + A * s; break;  // acoustic_pulse
      case 1: rho = 1 + A * s; u = 1.0; break;                   // entropy_wave
      case 2: rho = 1 + A * s; break;                            // density_pulse
      case 3: p = 1 + A * s; break;                              // pressure_pulse
      case 4: u = A * s; break;                                  // velocity_pulse
      default: break;
    }
    double* q = a.q + 3 * I.off;
    q[m] = rho * u;
    q[N + m] = rho;
    q[2 * N + m] = p / (g - 1) + 0.5 * rho * (u * u);
  }
}

__global__ void k2_sqerr_nodes(const Inst2D* inst, int ninst, BasisDev B, const double* u, const double* r, double* out,
                               long long NG) {
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < NG; n += (long long)gridDim.x * blockDim.x) {
    const Inst2D I = inst[find_inst(inst, ninst, n)];
    double c, x, y;
    node_coords2d(B, I, n - I.off, &c, &x, &y);
    const double d = u[n] - r[n];
    out[n] = c * (d * d);
  }
}

__global__ void k_sum_fixed(const double* f, long long n, double* out) {
  __shared__ double s[256];
  double acc = 0.0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) acc += f[i];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = s[0];
}

int grid_nodes(long long n) { return (int)std::min<long long>((n + 255) / 256, 152LL * 16); }

// Reference defaults of the builders' keyword arguments (initial_conditions.jl).
void default_prm(int type, double* prm) {
  std::memset(prm, 0, 15 * sizeof(double));
  if (type == 0) { prm[0] = 1.0; prm[1] = 1.0; prm[2] = 1.0; prm[3] = 1.0; }
  if (type == 1) { prm[0] = 5.0; prm[1] = 1.0; prm[2] = 1.0; }
  if (type == 3) { prm[0] = 1.0; prm[1] = 0.1; }
  if (type == 4) {
    const double d[11] = {0.05, 0.5, 0.25, 0.50, 0.09, 0.45, 0.60, 1.0, 0.45, 0.40, -1.0};
    std::memcpy(prm, d, sizeof(d));
  }
}
}  // namespace

int ic2d_param_count(int type) {
  switch (type) {
    case 0: return 4;
    case 1: return 3;
    case 2: return 0;
    case 3: return 2;
    case 4: return 11;
    case 5: return 15;
    default: throw Error(1, "Unknown IC type");
  }
}

void build_ic2d(Ctx& c, const Plan2D& P, int type, const double* amps, const double* params, double* const q[4]) {
  const int np_ = ic2d_param_count(type);
  const int ni = (int)P.inst.size();
  Ic2DArgs a;
  std::memset(&a, 0, sizeof(a));
  a.inst = P.d_inst; a.ninst = ni; a.B = P.B; a.type = type; a.NG = P.NG;
  default_prm(type, a.prm);
  if (params) std::memcpy(a.prm, params, np_ * sizeof(double));
  if (type == 5 && !(a.prm[2] >= 1 && a.prm[2] <= 4)) throw Error(1, "multi-blast IC needs 1..4 blasts (params[2])");
  for (int v = 0; v < 4; ++v) a.q[v] = q[v];
  double* d_amps = c.ws.dbl("ic:amps", ni);
  cuda_check(cudaMemcpyAsync(d_amps, amps, sizeof(double) * ni, cudaMemcpyHostToDevice, c.stream), "amps");
  a.amps = d_amps;
  std::vector<double> tab;
  if (type == 4) {
    // the enthalpy-defect table per instance (its circulation depends on gamma), trapezoid rule from r_max down
    tab.assign((size_t)ni * OSEEN_TAB, 0.0);
    for (int i = 0; i < ni; ++i) {
      const double g = P.inst[i].gamma, a_core = a.prm[0], r_max = 2.0 * P.inst[i].lx;
      const double Gam = a.prm[1] * std::sqrt(g) * 2 * kPi * a_core / 0.6383;
      const double pref = (Gam / (2 * kPi)) * (Gam / (2 * kPi));
      double* D = tab.data() + (size_t)i * OSEEN_TAB;
      double acc = 0.0;
      for (int k = OSEEN_TAB - 2; k >= 0; --k) {
        const double s1 = r_max * k / (OSEEN_TAB - 1), s2 = r_max * (k + 1) / (OSEEN_TAB - 1);
        const double e1 = 1.0 - std::exp(-(s1 * s1) / (a_core * a_core));
        const double e2 = 1.0 - std::exp(-(s2 * s2) / (a_core * a_core));
        const double f1 = s1 < 1e-12 ? 0.0 : (e1 * e1) / (s1 * s1 * s1);
        const double f2 = (e2 * e2) / (s2 * s2 * s2);
        acc += 0.5 * (f1 + f2) * (s2 - s1);
        D[k] = pref * acc;
      }
    }
    double* d_tab = c.ws.dbl("ic:tab", tab.size());
    cuda_check(cudaMemcpyAsync(d_tab, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice, c.stream), "table");
    a.tables = d_tab;
  }
  {
    LaunchScope ls(c, KID_OTHER);
    k2_build_ic<<<grid_nodes(P.NG), 256, 0, c.stream>>>(a);
  }
  cuda_check(cudaStreamSynchronize(c.stream), "sync");  // the host table must outlive the copy
}

void build_ic1d(Ctx& c, const Plan1D& P, int type, const double* amps, double* q) {
  if (type < 0 || type > 4) throw Error(1, "Unknown IC type");
  const int ni = (int)P.inst.size();
  Ic1DArgs a;
  std::memset(&a, 0, sizeof(a));
  a.inst = P.d_inst; a.ninst = ni; a.B = P.B; a.type = type; a.q = q; a.NG = P.NG;
  double* d_amps = c.ws.dbl("ic:amps1", ni);
  cuda_check(cudaMemcpyAsync(d_amps, amps, sizeof(double) * ni, cudaMemcpyHostToDevice, c.stream), "amps");
  a.amps = d_amps;
  {
    LaunchScope ls(c, KID_OTHER);
    k1_build_ic<<<grid_nodes(P.NG), 256, 0, c.stream>>>(a);
  }
  cuda_check(cudaStreamSynchronize(c.stream), "sync");
}

double l2_error2d(Ctx& c, const Plan2D& P, const double* u, const double* r) {
  double* f = c.ws.dbl("ic:sq", P.NG);
  double* out = c.ws.dbl("ic:sum", 1);
  {
    LaunchScope ls(c, KID_OTHER);
    k2_sqerr_nodes<<<grid_nodes(P.NG), 256, 0, c.stream>>>(P.d_inst, (int)P.inst.size(), P.B, u, r, f, P.NG);
  }
  {
    LaunchScope ls(c, KID_OTHER);
    k_sum_fixed<<<1, 256, 0, c.stream>>>(f, P.NG, out);
  }
  double h = 0.0;
  cuda_check(cudaMemcpyAsync(&h, out, sizeof(double), cudaMemcpyDeviceToHost, c.stream), "readback");
  cuda_check(cudaStreamSynchronize(c.stream), "sync");
  return std::sqrt(h);
}

}  // namespace igrgpu
