// Build shim: the sparse (SuiteSparse) entry points of the xerus reference,
// replaced by functions that throw. The oracle builds every operator core
// densely, so the dense path it exercises never calls these.
#include <stdexcept>
#include <xerus/cholmod_wrapper.h>

namespace xerus { namespace internal {
[[noreturn]] static void sparse_unavailable() { throw std::runtime_error("sparse (SuiteSparse) path is not built into this oracle"); }
void CholmodSparse::matrix_matrix_product(std::map<size_t, double>&, const size_t, const size_t, const double,
                                          const std::map<size_t, double>&, const bool, const size_t,
                                          const std::map<size_t, double>&, const bool) { sparse_unavailable(); }
void CholmodSparse::solve_sparse_rhs(std::map<size_t, double>&, size_t, const std::map<size_t, double>&, const bool,
                                     const std::map<size_t, double>&, size_t) { sparse_unavailable(); }
void CholmodSparse::solve_dense_rhs(double*, size_t, const std::map<size_t, double>&, const bool, const double*, size_t) { sparse_unavailable(); }
std::tuple<std::map<size_t, double>, std::map<size_t, double>, size_t>
CholmodSparse::qc(const std::map<size_t, double>&, const bool, size_t, size_t, bool) { sparse_unavailable(); }
std::tuple<std::map<size_t, double>, std::map<size_t, double>, size_t>
CholmodSparse::cq(const std::map<size_t, double>&, const bool, size_t, size_t, bool) { sparse_unavailable(); }
}}
