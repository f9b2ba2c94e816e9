// Adjoint launch wrappers (kernels_adjoint.cu); periodic domain, FP64.
#pragma once

#include "kernels.h"

namespace afmib {

// (ou, ov, ow) (+)= N'(u)^T (lu, lv, lw), the transposed Jacobian of the advection term
void launch_advect_adjoint(const Dims& d, double* ou, double* ov, double* ow, const double* u, const double* v,
                           const double* w, const double* lu, const double* lv, const double* lw, int acc,
                           cudaStream_t s);

// gX[k][a] += scale * sum_c g[c][k] * sum_faces d/dX_a (phi/n)^3 F_c(face)
void launch_marker_grad(const Dims& d, int M, const double* X, const double* g, const double* Fu, const double* Fv,
                        const double* Fw, double scale, double* gX, cudaStream_t s);

// gX += k K^T lamG (symmetric lists); dk_part[i] = lamG_i . (K X)_i
// gX += -kb L (L lamG): the bending term of the marker-force adjoint
// (lamG per component, gX like X; Z: 3M doubles of workspace)
void launch_bending_adjoint(int M, const int* ns, const int* ni, double kb, const double* lamG, double* Z, double* gX,
                            cudaStream_t s);
void launch_springs_adjoint(int M, const double* X, const int* ns, const int* ni, double kspring, const double* lamG,
                            double* gX, double* dk_part, cudaStream_t s);

// soa[c*M + k] = c0 * aos[3k + c]; aos[3k + c] += c0 * soa[c*M + k]
void launch_aos_to_soa(int M, const double* aos, double* soa, double c0, cudaStream_t s);
void launch_soa_add_aos(int M, const double* soa, double* aos, double c0, cudaStream_t s);

}  // namespace afmib
