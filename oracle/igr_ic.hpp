// ORACLE — test infrastructure only (see igr_common.hpp for the parity status).
// Initial-condition builders and the quadrature L2 error, restated from
// IGR_adjoints_2d/initial_conditions.jl:15-232 and
// IGR_adjoints_1d/initial_conditions.jl:94-204 (expression by expression).
#pragma once
#include "igr1d.hpp"

namespace igr {

enum IC2D { IC2_CONSTANT = 0, IC2_ISENTROPIC_VORTEX = 1, IC2_TAYLOR_GREEN = 2, IC2_SEDOV_BLAST = 3, IC2_OSEEN_PAIR_BLAST = 4,
            IC2_MULTI_BLAST = 5 };
enum IC1D { IC1_ACOUSTIC_PULSE = 0, IC1_ENTROPY_WAVE = 1, IC1_DENSITY_PULSE = 2, IC1_PRESSURE_PULSE = 3, IC1_VELOCITY_PULSE = 4 };

// Enthalpy-defect table of build_oseen_pair_blast_ic! (initial_conditions.jl:
// 182-194): D(r_i) = (Gamma/2pi)^2 int_{r_i}^{r_max} (1 - e^{-s^2/a^2})^2 / s^3 ds
// by the trapezoid rule on n_tab equispaced points of [0, r_max].
inline std::vector<double> oseen_defect_table(double Gamma, double a_core, double r_max, int n_tab) {
  const double pi = 3.14159265358979323846;
  std::vector<double> D(n_tab, 0.0);
  const double pref = (Gamma / (2 * pi)) * (Gamma / (2 * pi));
  double acc = 0.0;
  for (int i = n_tab - 2; i >= 0; --i) {
    const double s1 = r_max * i / (n_tab - 1), s2 = r_max * (i + 1) / (n_tab - 1);
    const double e1 = 1.0 - std::exp(-(s1 * s1) / (a_core * a_core));
    const double e2 = 1.0 - std::exp(-(s2 * s2) / (a_core * a_core));
    const double f1 = s1 < 1e-12 ? 0.0 : (e1 * e1) / (s1 * s1 * s1);
    const double f2 = (e2 * e2) / (s2 * s2 * s2);
    acc += 0.5 * (f1 + f2) * (s2 - s1);
    D[i] = pref * acc;
  }
  return D;
}

inline double oseen_defect(const std::vector<double>& D, double r, double r_max) {
  const int n_tab = (int)D.size();
  if (r >= r_max) return 0.0;
  const double t = r / r_max * (n_tab - 1) + 1;
  int i = (int)std::floor(t);
  i = std::min(std::max(i, 1), n_tab - 1);
  const double w = t - i;
  return (1 - w) * D[i - 1] + w * D[i];
}

// One 2D builder at node (x, y). prm: constant (rho0, ux0, uy0, p0);
// isentropic vortex (beta, ux0, uy0); Sedov (p_bg, sigma); Oseen pair (a_core,
// M_star, blast_xc, blast_yc, sigma, xc1, yc1, sign1, xc2, yc2, sign2).
inline void ic2d_node(int type, double x, double y, double Lx, double Ly, double g, double A, const double* prm,
                      const std::vector<double>& table, double q[4]) {
  const double pi = 3.14159265358979323846;
  double rho = 1.0, ux = 0.0, uy = 0.0, p = 1.0;
  switch (type) {
    case IC2_CONSTANT: rho = prm[0]; ux = prm[1]; uy = prm[2]; p = prm[3]; break;
    case IC2_ISENTROPIC_VORTEX: {  // init_isentropic_vortex, :39-67
      const double beta = prm[0];
      const double dx = x - Lx / 2, dy = y - Ly / 2;
      const double r2 = dx * dx + dy * dy;
      const double ef = std::exp((1 - r2) / 2);
      const double du = -dy * (beta / (2 * pi)) * ef;
      const double dv = dx * (beta / (2 * pi)) * ef;
      const double dT = -(g - 1) * (beta * beta) / (8 * g * (pi * pi)) * std::exp(1 - r2);
      rho = std::pow(1 + dT, 1 / (g - 1));
      ux = prm[1] + du;
      uy = prm[2] + dv;
      p = std::pow(rho, g);
      break;
    }
    case IC2_TAYLOR_GREEN: {  // build_taylor_green_ic!, :105-121
      const double cx = 2 * pi * x / Lx, cy = 2 * pi * y / Ly;
      ux = A * std::sin(cx) * std::cos(cy);
      uy = -A * std::cos(cx) * std::sin(cy);
      break;
    }
    case IC2_SEDOV_BLAST: {  // build_sedov_blast_ic!, :136-150
      const double dx = x - Lx / 2, dy = y - Ly / 2;
      const double r2 = dx * dx + dy * dy;
      p = prm[0] + A * std::exp(-r2 / (prm[1] * prm[1]));
      break;
    }
    case IC2_OSEEN_PAIR_BLAST: {  // build_oseen_pair_blast_ic!, :175-231
      const double a_core = prm[0], M_star = prm[1];
      const double L = Lx;
      const double Gam = M_star * std::sqrt(g) * 2 * pi * a_core / 0.6383;
      const double r_max = 2.0 * L;
      double h = g / (g - 1);
      for (int k = 0; k < 2; ++k) {
        const double xc = prm[5 + 3 * k], yc = prm[6 + 3 * k], sgn = prm[7 + 3 * k];
        const double Gk = sgn * Gam;
        for (int sx = -1; sx <= 1; ++sx)
          for (int sy = -1; sy <= 1; ++sy) {
            const double dx = x - (xc + sx * L), dy = y - (yc + sy * L);
            const double r2 = dx * dx + dy * dy;
            if (r2 < 1e-24) continue;
            const double vr = Gk / (2 * pi * r2) * (1.0 - std::exp(-r2 / (a_core * a_core)));
            ux += -vr * dy;
            uy += vr * dx;
          }
        double dx = x - xc, dy = y - yc;
        dx -= L * std::nearbyint(dx / L);
        dy -= L * std::nearbyint(dy / L);
        h -= oseen_defect(table, std::sqrt(dx * dx + dy * dy), r_max);
      }
      const double p_vort = std::pow((g - 1) * h / g, g / (g - 1));
      rho = std::pow(p_vort, 1.0 / g);
      const double r2b = (x - prm[2]) * (x - prm[2]) + (y - prm[3]) * (y - prm[3]);
      p = p_vort + A * std::exp(-r2b / (prm[4] * prm[4]));
      break;
    }
    case IC2_MULTI_BLAST: {
      // the paper scripts' several-blast state (2d/paper_scripts/generate_otd_refinement_sedov_data.jl:72-86):
      // rho = 1, u = 0, p = p_bg + sum_k A_k exp(-r_k^2 / sigma^2); prm = (p_bg, sigma, n, x_1, y_1, A_1, ...),
      // blast 1's amplitude is A (the differentiated parameter)
      const int nb = (int)prm[2];
      double pv = prm[0];
      for (int k = 0; k < nb; ++k) {
        const double r2 = (x - prm[3 + 3 * k]) * (x - prm[3 + 3 * k]) + (y - prm[4 + 3 * k]) * (y - prm[4 + 3 * k]);
        pv += (k == 0 ? A : prm[5 + 3 * k]) * std::exp(-r2 / (prm[1] * prm[1]));
      }
      p = pv;
      break;
    }
    default: throw std::invalid_argument("Unknown IC type");
  }
  q[2] = rho;
  q[0] = rho * ux;
  q[1] = rho * uy;
  q[3] = p / (g - 1) + 0.5 * rho * (ux * ux + uy * uy);
}

inline void build_ic2d(const Grid2D& G, int type, double g, double A, const double* prm, double* const q[4]) {
  std::vector<double> table;
  if (type == IC2_OSEEN_PAIR_BLAST) {
    const double pi = 3.14159265358979323846;
    const double Gam = prm[1] * std::sqrt(g) * 2 * pi * prm[0] / 0.6383;
    table = oseen_defect_table(Gam, prm[0], 2.0 * G.m.Lx, 4000);
  }
  for (int ey = 0; ey < G.m.Ney; ++ey) for (int ex = 0; ex < G.m.Nex; ++ex)
    for (int j = 0; j < G.np; ++j) for (int i = 0; i < G.np; ++i) {
      const size_t n = G.id(i, j, ex, ey);
      double v[4];
      ic2d_node(type, node_x(G.b, G.m, i, ex), node_y(G.b, G.m, j, ey), G.m.Lx, G.m.Ly, g, A, prm, table, v);
      for (int c = 0; c < 4; ++c) q[c][n] = v[c];
    }
}

// IGR_adjoints_1d/initial_conditions.jl:94-204: rho, u, p from s = sin(2 pi x / L).
inline void build_ic1d(const Grid1D& G, int type, double g, double A, double* const q[3]) {
  const double pi = 3.14159265358979323846;
  for (int e = 0; e < G.m.Ne; ++e)
    for (int i = 0; i < G.np; ++i) {
      const size_t n = G.id(i, e);
      const double s = std::sin(2 * pi * G.x(i, e) / G.m.L);
      double rho = 1.0, u = 0.0, p = 1.0;
      switch (type) {
        case IC1_ACOUSTIC_PULSE: rho = 1 + A * s; u = A * s; p = 1 + A * s; break;
        case IC1_ENTROPY_WAVE: rho = 1 + A * s; u = 1.0; break;
        case IC1_DENSITY_PULSE: rho = 1 + A * s; break;
        case IC1_PRESSURE_PULSE: p = 1 + A * s; break;
        case IC1_VELOCITY_PULSE: u = A * s; break;
        default: throw std::invalid_argument("Unknown IC type");
      }
      q[1][n] = rho;
      q[0][n] = rho * u;
      q[2][n] = p / (g - 1) + 0.5 * rho * (u * u);
    }
}

// l2_error, IGR_adjoints_2d/initial_conditions.jl:74-87 (and the 1D form).
inline double l2_error2d(const Grid2D& G, const double* u, const double* r) {
  double e2 = 0.0;
  for (int ey = 0; ey < G.m.Ney; ++ey) for (int ex = 0; ex < G.m.Nex; ++ex)
    for (int j = 0; j < G.np; ++j) for (int i = 0; i < G.np; ++i) {
      const size_t n = G.id(i, j, ex, ey);
      e2 += G.b.w[i] * G.b.w[j] * (G.m.Jx * G.m.Jy) * ((u[n] - r[n]) * (u[n] - r[n]));
    }
  return std::sqrt(e2);
}

}  // namespace igr
