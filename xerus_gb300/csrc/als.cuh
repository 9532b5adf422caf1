// ALS / DMRG for SPD operators on device-resident TTs: environment stacks,
// the local operator as a chain of strided GEMMs, a persistent conjugate-
// gradient local solver, and the sweep driver of ALSVariant::solve.
#pragma once

#include <vector>

#include "engine.cuh"

namespace xtt {

// The local operator y = (L . A_k [. A_k+1] . R) x of the SPD sweep
// (src/xerus/algorithms/als.cpp:383-401) as 3 (one site) or 4 (two sites)
// GEMM stages; g[0].B is the input vector, g[ns-1].C the output.
template <class T>
struct MatvecPlan {
	int ns = 0;
	long long n = 0;  // local dimension
	Gemm<T> g[4];
};

struct LocalShape {
	int sites = 1;
	int ra = 1, rb = 1;        // x ranks around the block
	int n1 = 1, n2 = 1;        // mode sizes
	int K0 = 1, K1 = 1, K2 = 1; // operator ranks (K2 used for two sites)
	long long dim() const { return (long long)ra * n1 * (sites == 2 ? n2 : 1) * rb; }
};

template <class T>
MatvecPlan<T> make_matvec_plan(const LocalShape& s, const T* L, const T* A1, const T* A2, const T* R, T* t1, T* t2,
                               T* t3);
size_t matvec_tmp_elems(const LocalShape& s, int stage);  // elements of intermediate `stage` (0..2)

struct CgResult {
	int iterations = 0;
	int refinements = 0;
	double rel_residual = 0;
};

// Solves the local SPD system M x = b in place (x holds the initial guess).
// FP64: CG to ||r|| <= tol ||b||. Mixed: FP32 CG corrections with FP64 residuals.
CgResult local_solve(Context& c, const LocalShape& s, const double* L, const double* A1, const double* A2,
                     const double* R, const double* b, double* x, double tol, int max_iter, int precision);

// The same solve in one thread-block cluster with every operand in shared
// memory (cg_cluster.cu); false when the system does not fit, in which case
// nothing was launched.
bool cluster_local_solve(Context& c, const LocalShape& s, const double* L, const double* A1, const double* A2,
                         const double* R, const double* b, double* x, double tol, int max_iter, int precision);

// y = M x once (FP64), host-launched chain.
void local_matvec(Context& c, const LocalShape& s, const double* L, const double* A1, const double* A2,
                  const double* R, const double* x, double* y);

struct AlsOptions {
	int sites = 1;
	int local_solver = 0;  // 0 exact (CG), 1 ASD step
	bool preserve_core_position = true;
	int precision = 0;
	int64_t num_half_sweeps = 0;
	double convergence_epsilon = 1e-6;
	double local_tolerance = 1e-13;
	int64_t local_max_iterations = 0;
	double residual_target = 0;
	bool record_residuals = false;
	int max_rank = 0;
	double svd_epsilon = 0;
	bool exact_environment = false;  // 2 sites: push core k+1 (not k) in decreasing sweeps
};

struct AlsReport {
	double energy = 0, residual = -1;
	int64_t half_sweeps = 0, micro_steps = 0, local_iterations = 0, refinements = 0;
	std::vector<double> residuals, energies;
	std::vector<int64_t> flags;
};

AlsReport als(const Tensor& A, Tensor& x, const Tensor& b, const AlsOptions& o);

// J(x) = <x,Ax> - 2<x,b> and dJ/dX_k for every core.
double als_energy_gradient(const Tensor& A, const Tensor& x, const Tensor& b, std::vector<double>& grad);

}  // namespace xtt
