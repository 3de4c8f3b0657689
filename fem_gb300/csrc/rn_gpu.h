// rn_gpu.h - device kernels of the reflective Newton step (internal; rn_kernels.cu).
#pragma once

namespace lina {
namespace rn {

// bound constraints on the device: constraint i acts on unknown idx[i], bounds lo[i] and up[i]
// (NaN = no bound)
struct Bounds {
    int nb = 0;
    int* idx = nullptr;
    double* lo = nullptr;
    double* up = nullptr;
};

bool set_DJ(long n, const Bounds& b, const double* G, const double* X, double* D, double* J);
bool pmult(double* a, const double* b, long n);          // a *= b elementwise
bool reflect(const Bounds& b, double* X);                // fold X back into the box
bool snap(const Bounds& b, double* X, double eps);       // X = bound where |X - bound| < eps
int at_boundary(const Bounds& b, const double* X);       // 1 if some |X - bound| < 1e-30, -1 on error

}  // namespace rn
}  // namespace lina
