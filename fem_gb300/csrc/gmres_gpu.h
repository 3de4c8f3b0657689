// gmres_gpu.h - restarted GMRES on device vectors (internal; gpu_gmres.cu).
#pragma once

#include <functional>

namespace lina {
namespace gm {

// y = op(x) on device vectors of the system's length; an empty Op is the identity
using Op = std::function<bool(const double* x, double* y)>;

struct Result {
    int iter = 0, rcode = 0, nomatvec = 0, noprecl = 0, noprecr = 0;
    double precision = 0.0, residuum = 0.0;
};

// M y = b with M = preconl A preconr from the initial y (device vectors); see gpu_gmres.cu.
// Returns false on a device failure; res.rcode follows the ITLIN_INFO codes (0, 1, 2).
bool solve(long n, double* y, const double* b, const Op& matvec, const Op& preconr, const Op& preconl, double tol,
           int i_max, int max_iter, bool check_each, Result& res);

}  // namespace gm
}  // namespace lina
