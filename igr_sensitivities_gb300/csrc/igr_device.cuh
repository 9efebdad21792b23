// Device-side types shared by the 2D and 1D kernel families.
//
// Layout in HBM: every field (state variable, coefficient, tape slot) is one
// contiguous FP64 array over all instances of a batch group, instance-major.
// Inside an instance the node order is the reference's Julia column-major
// order, (n_p, n_p, N_ex, N_ey) with the x-node fastest
// (IGR_adjoints_2d/mesh.jl:85-88): the NP*NP nodes of an element are
// contiguous (128 B for P3), so each element is one aligned block.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace igrgpu {

constexpr int MAXNP = 5;  // p <= 4

// DG basis constants (IGR_adjoints_2d/basis.jl:7-12), passed by value as a
// kernel parameter (constant bank, broadcast reads).
struct BasisDev {
  int np;
  double D[MAXNP][MAXNP];   // D[i][k] = l_k'(xi_i)
  double w[MAXNP];          // LGL weights
  double xi[MAXNP];         // LGL nodes (node coordinates for windowed objectives)
  double W2[MAXNP][MAXNP];  // w_i * D[i][k]^2 (diagonal of the stiffness term)
  double cheb_theta, cheb_delta, cheb_sigma;  // elliptic.jl:373-378
  double hw;                // -1 / (2 w_0): SIP face coefficient factor
  double iw0, iwL;          // 1 / w_0, 1 / w_L
};

// One problem instance of a batch (2D): mesh, physics parameters and where
// its nodes start in every field array.
struct Inst2D {
  long long off;    // first node of this instance in every field
  int nex, ney;
  double lx, ly, dx, dy, jx, jy;
  double gamma, alpha, dt;
  // reciprocals precomputed on the host (an FP64 divide costs ~9 FMA slots)
  double ijx, ijy, idx, idy, ialpha;
};

struct Inst1D {
  long long off;
  int ne, pad;
  double dx, jac;
  double gamma, alpha, dt;
};

// A tile of TX x TY elements of one instance; blocks map 1:1 onto tiles.
struct Tile2D { int inst, ex0, ey0, pad; };

// Status word shared by the kernels and the host (device memory).
enum : int { DEV_OK = 0, DEV_NONFINITE = 1 };

__device__ __forceinline__ void flag_nonfinite(int* status) {
  if (status) atomicOr(status, DEV_NONFINITE);
}

}  // namespace igrgpu
