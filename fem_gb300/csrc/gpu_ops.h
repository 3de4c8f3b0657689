// gpu_ops.h - device vector toolkit for the LinA drop-in solvers (internal).
//
// The reference's Krylov loops (pcg, BiCGStab_solve) are restated in
// lina_api.cpp on device vectors; these helpers run their BLAS-1 steps on the
// GPU (one stream, deterministic single-pass reductions) and stage vectors for
// callbacks the caller installs.
#pragma once

namespace lina {
namespace dev {

bool ready();                                      // context created (creates on first use)
double* alloc(long n);                             // FP64 device vector, nullptr on failure
void release(void* p);
bool h2d(double* d, const double* h, long n);
bool h2d_bytes(void* d, const void* h, long bytes);
bool d2h(double* h, const double* d, long n);
bool d2d(double* d, const double* s, long n);
bool zero(double* d, long n);
double dot(const double* a, const double* b, long n);  // NaN on failure
bool axpy(double* y, double a, const double* x, long n);  // y += a x
bool scal(double* x, double a, long n);                   // x *= a
bool xpay(double* y, const double* x, double a, long n);  // y = x + a y
bool sync();
void* stream();                                    // the cudaStream_t used by these helpers
void set_error(const char* msg);                   // text returned by lina_gpu_last_error()

}  // namespace dev
}  // namespace lina
