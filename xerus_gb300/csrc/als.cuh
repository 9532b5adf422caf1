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
	__host__ __device__ long long dim() const { return (long long)ra * n1 * (sites == 2 ? n2 : 1) * rb; }
};

__host__ __device__ inline size_t matvec_tmp_elems(const LocalShape& s, int stage) {
	const size_t ra = s.ra, rb = s.rb, n1 = s.n1, n2 = s.n2, K0 = s.K0, K1 = s.K1, K2 = s.K2;
	if (s.sites == 1) {
		if (stage == 0) return ra * K0 * n1 * rb;  // S1 (a, k, j, b')
		if (stage == 1) return ra * n1 * K1 * rb;  // S2 (a, i, k', b')
		return 1;
	}
	if (stage == 0) return ra * K0 * n1 * n2 * rb;  // S1 (a, k0, j1, j2, b')
	if (stage == 1) return ra * n1 * K1 * n2 * rb;  // S2 (a, i1, k1, j2, b')
	return ra * n1 * n2 * K2 * rb;                  // S3 (a, i1, i2, k2, b')
}

// y(a,i,b) = sum L(a,k,a') A(k,i,j,k') R(b,k',b') x(a',j,b')  (1 site), and the
// analogous 2-site product; row index (a, i.., b), column index (a', j.., b').
template <class T>
__host__ __device__ MatvecPlan<T> make_matvec_plan(const LocalShape& s, const T* L, const T* A1, const T* A2, const T* R, T* t1, T* t2,
                               T* t3) {
	MatvecPlan<T> p;
	p.n = s.dim();
	const long long ra = s.ra, rb = s.rb, n1 = s.n1, n2 = s.n2, K0 = s.K0, K1 = s.K1, K2 = s.K2;
	const long long nL = ra * K0 * ra, nA1 = K0 * n1 * n1 * K1, nA2 = K1 * n2 * n2 * K2;
	const long long nR = rb * (s.sites == 2 ? K2 : K1) * rb, nx = p.n;
	const long long n0 = (long long)matvec_tmp_elems(s, 0), nt1 = (long long)matvec_tmp_elems(s, 1),
	                nt2 = (long long)matvec_tmp_elems(s, 2);
	if (s.sites == 1) {
		p.ns = 3;
		Gemm<T>& g1 = p.g[0];  // S1((a,k),(j,b')) = L((a,k),a') x(a',(j,b'))
		g1.M = int(ra * K0); g1.N = int(n1 * rb); g1.K = int(ra);
		g1.A = L; g1.sAm = ra; g1.sAk = 1;
		g1.sBk = n1 * rb; g1.sBn = 1;
		g1.C = t1; g1.sCm = n1 * rb; g1.sCn = 1;
		g1.lens(nL, nx, n0);
		Gemm<T>& g2 = p.g[1];  // per a: S2(a,i,k',b') = sum_(k,j) S1(a,k,j,b') A(k,i,j,k')
		g2.batch = int(ra); g2.M = int(rb); g2.N = int(n1 * K1); g2.Ni = int(K1); g2.K = int(K0 * n1); g2.Ki = int(n1);
		g2.A = t1; g2.sAb = K0 * n1 * rb; g2.sAm = 1; g2.sAko = n1 * rb; g2.sAk = rb;
		g2.B = A1; g2.sBko = n1 * n1 * K1; g2.sBk = K1; g2.sBno = n1 * K1; g2.sBn = 1;
		g2.C = t2; g2.sCb = n1 * K1 * rb; g2.sCm = 1; g2.sCno = K1 * rb; g2.sCn = rb;
		g2.lens(n0, nA1, nt1);
		Gemm<T>& g3 = p.g[2];  // y((a,i),b) = sum_(k',b') S2((a,i),(k',b')) R(b,(k',b'))
		g3.M = int(ra * n1); g3.N = int(rb); g3.K = int(K1 * rb);
		g3.A = t2; g3.sAm = K1 * rb; g3.sAk = 1;
		g3.B = R; g3.sBk = 1; g3.sBn = K1 * rb;
		g3.sCm = rb; g3.sCn = 1;
		g3.lens(nt1, nR, nx);
	} else {
		p.ns = 4;
		Gemm<T>& g1 = p.g[0];  // S1((a,k0),(j1,j2,b'))
		g1.M = int(ra * K0); g1.N = int(n1 * n2 * rb); g1.K = int(ra);
		g1.A = L; g1.sAm = ra; g1.sAk = 1;
		g1.sBk = n1 * n2 * rb; g1.sBn = 1;
		g1.C = t1; g1.sCm = n1 * n2 * rb; g1.sCn = 1;
		g1.lens(nL, nx, n0);
		Gemm<T>& g2 = p.g[1];  // per a: S2(a,i1,k1,(j2,b')) = sum_(k0,j1) S1(a,k0,j1,(j2,b')) A1(k0,i1,j1,k1)
		g2.batch = int(ra); g2.M = int(n2 * rb); g2.N = int(n1 * K1); g2.Ni = int(K1); g2.K = int(K0 * n1); g2.Ki = int(n1);
		g2.A = t1; g2.sAb = K0 * n1 * n2 * rb; g2.sAm = 1; g2.sAko = n1 * n2 * rb; g2.sAk = n2 * rb;
		g2.B = A1; g2.sBko = n1 * n1 * K1; g2.sBk = K1; g2.sBno = n1 * K1; g2.sBn = 1;
		g2.C = t2; g2.sCb = n1 * K1 * n2 * rb; g2.sCm = 1; g2.sCno = K1 * n2 * rb; g2.sCn = n2 * rb;
		g2.lens(n0, nA1, nt1);
		Gemm<T>& g3 = p.g[2];  // per (a,i1): S3(a,i1,i2,k2,b') = sum_(k1,j2) S2(a,i1,k1,j2,b') A2(k1,i2,j2,k2)
		g3.batch = int(ra * n1); g3.M = int(rb); g3.N = int(n2 * K2); g3.Ni = int(K2); g3.K = int(K1 * n2); g3.Ki = int(n2);
		g3.A = t2; g3.sAb = K1 * n2 * rb; g3.sAm = 1; g3.sAko = n2 * rb; g3.sAk = rb;
		g3.B = A2; g3.sBko = n2 * n2 * K2; g3.sBk = K2; g3.sBno = n2 * K2; g3.sBn = 1;
		g3.C = t3; g3.sCb = n2 * K2 * rb; g3.sCm = 1; g3.sCno = K2 * rb; g3.sCn = rb;
		g3.lens(nt1, nA2, nt2);
		Gemm<T>& g4 = p.g[3];  // y((a,i1,i2),b) = sum_(k2,b') S3((a,i1,i2),(k2,b')) R(b,(k2,b'))
		g4.M = int(ra * n1 * n2); g4.N = int(rb); g4.K = int(K2 * rb);
		g4.A = t3; g4.sAm = K2 * rb; g4.sAk = 1;
		g4.B = R; g4.sBk = 1; g4.sBn = K2 * rb;
		g4.sCm = rb; g4.sCn = 1;
		g4.lens(nt2, nR, nx);
	}
	return p;
}


// Environment pushes of the SPD sweep as GEMM chains (descriptors only, so the
// host driver and the batched persistent kernel run identical contractions).
struct GemmChain {
	int ns = 0;
	Gemm<double> g[3];
};

// L'(c1,c2,c3) = sum L(a1,a2,a3) x(a1,i,c1) A(a2,i,j,c2) x(a3,j,c3)       (als.cpp:184-200, 247)
// scratch: s1 K r n r1, s2 r r1 n K1
__host__ __device__ inline GemmChain plan_push_left_op(const double* L, const double* x, const double* A, double* out,
                                                      double* s1, double* s2, long long r, long long K, long long n,
                                                      long long r1, long long K1) {
	GemmChain ch;
	ch.ns = 3;
	Gemm<double>& p1 = ch.g[0];  // S1((a2,a3),(i,c1)) = sum_a1 L(a1,(a2,a3)) x(a1,(i,c1))
	p1.M = int(K * r); p1.N = int(n * r1); p1.K = int(r);
	p1.A = L; p1.sAm = 1; p1.sAk = K * r;
	p1.B = x; p1.sBk = n * r1; p1.sBn = 1;
	p1.C = s1; p1.sCm = n * r1; p1.sCn = 1;
	p1.lens(r * K * r, r * n * r1, K * r * n * r1);
	Gemm<double>& p2 = ch.g[1];  // per a3: S2(a3,c1,(j,c2)) = sum_(a2,i) S1(a2,a3,i,c1) A((a2,i),(j,c2))
	p2.batch = int(r); p2.M = int(r1); p2.N = int(n * K1); p2.K = int(K * n); p2.Ki = int(n);
	p2.A = s1; p2.sAb = n * r1; p2.sAm = 1; p2.sAko = r * n * r1; p2.sAk = r1;
	p2.B = A; p2.sBko = n * n * K1; p2.sBk = n * K1; p2.sBn = 1;
	p2.C = s2; p2.sCb = r1 * n * K1; p2.sCm = n * K1; p2.sCn = 1;
	p2.lens(K * r * n * r1, K * n * n * K1, r * r1 * n * K1);
	Gemm<double>& p3 = ch.g[2];  // L'((c1,c2),c3) = sum_(a3,j) S2(a3,c1,j,c2) x((a3,j),c3)
	p3.M = int(r1 * K1); p3.Mi = int(K1); p3.N = int(r1); p3.K = int(r * n); p3.Ki = int(n);
	p3.A = s2; p3.sAmo = n * K1; p3.sAm = 1; p3.sAko = r1 * n * K1; p3.sAk = K1;
	p3.B = x; p3.sBko = n * r1; p3.sBk = r1; p3.sBn = 1;
	p3.C = out; p3.sCmo = K1 * r1; p3.sCm = r1; p3.sCn = 1;
	p3.lens(r * r1 * n * K1, r * n * r1, r1 * K1 * r1);
	return ch;
}

// R'(a1,a2,a3) = sum x(a1,i,c1) A(a2,i,j,c2) x(a3,j,c3) R(c1,c2,c3)       (als.cpp:239)
// scratch: s1 r n r1 K1, s2 r K n r1
__host__ __device__ inline GemmChain plan_push_right_op(const double* R, const double* x, const double* A, double* out,
                                                       double* s1, double* s2, long long r, long long K, long long n,
                                                       long long r1, long long K1) {
	GemmChain ch;
	ch.ns = 3;
	Gemm<double>& q1 = ch.g[0];  // S1((a3,j),(c1,c2)) = sum_c3 x((a3,j),c3) R((c1,c2),c3)
	q1.M = int(r * n); q1.N = int(r1 * K1); q1.K = int(r1);
	q1.A = x; q1.sAm = r1; q1.sAk = 1;
	q1.B = R; q1.sBk = 1; q1.sBn = r1;
	q1.C = s1; q1.sCm = r1 * K1; q1.sCn = 1;
	q1.lens(r * n * r1, r1 * K1 * r1, r * n * r1 * K1);
	Gemm<double>& q2 = ch.g[1];  // per a3: S2(a3,(a2,i),c1) = sum_(j,c2) A((a2,i),(j,c2)) S1(a3,j,c1,c2)
	q2.batch = int(r); q2.M = int(K * n); q2.N = int(r1); q2.K = int(n * K1); q2.Ki = int(K1);
	q2.A = A; q2.sAm = n * K1; q2.sAko = K1; q2.sAk = 1;
	q2.B = s1; q2.sBb = n * r1 * K1; q2.sBko = r1 * K1; q2.sBk = 1; q2.sBn = K1;
	q2.C = s2; q2.sCb = K * n * r1; q2.sCm = r1; q2.sCn = 1;
	q2.lens(K * n * n * K1, r * n * r1 * K1, r * K * n * r1);
	Gemm<double>& q3 = ch.g[2];  // R'(a1,(a2,a3)) = sum_(i,c1) x(a1,(i,c1)) S2(a3,a2,(i,c1))
	q3.M = int(r); q3.N = int(K * r); q3.Ni = int(r); q3.K = int(n * r1);
	q3.A = x; q3.sAm = n * r1; q3.sAk = 1;
	q3.B = s2; q3.sBk = 1; q3.sBno = n * r1; q3.sBn = K * n * r1;
	q3.C = out; q3.sCm = K * r; q3.sCno = r; q3.sCn = 1;
	q3.lens(r * n * r1, r * K * n * r1, r * K * r);
	return ch;
}

// Lb'(c1,c2) = sum Lb(a1,a2) b(a1,i,c1) x(a2,i,c2)   (als.cpp:202-215, 250); scratch t: r n s1
__host__ __device__ inline GemmChain plan_push_left_rhs(const double* Lb, const double* bc, const double* x, double* out,
                                                       double* t, long long s, long long r, long long n, long long s1,
                                                       long long r1) {
	GemmChain ch;
	ch.ns = 2;
	Gemm<double>& u1 = ch.g[0];  // S1(a2,(i,c1)) = sum_a1 Lb(a1,a2) b(a1,(i,c1))
	u1.M = int(r); u1.N = int(n * s1); u1.K = int(s);
	u1.A = Lb; u1.sAm = 1; u1.sAk = r;
	u1.B = bc; u1.sBk = n * s1; u1.sBn = 1;
	u1.C = t; u1.sCm = n * s1; u1.sCn = 1;
	u1.lens(s * r, s * n * s1, r * n * s1);
	Gemm<double>& u2 = ch.g[1];  // Lb'(c1,c2) = sum_(a2,i) S1((a2,i),c1) x((a2,i),c2)
	u2.M = int(s1); u2.N = int(r1); u2.K = int(r * n);
	u2.A = t; u2.sAm = 1; u2.sAk = s1;
	u2.B = x; u2.sBk = r1; u2.sBn = 1;
	u2.C = out; u2.sCm = r1; u2.sCn = 1;
	u2.lens(r * n * s1, r * n * r1, s1 * r1);
	return ch;
}

// Rb'(a1,a2) = sum b(a1,i,c1) x(a2,i,c2) Rb(c1,c2)   (als.cpp:242); scratch t: r n s1
__host__ __device__ inline GemmChain plan_push_right_rhs(const double* Rb, const double* bc, const double* x, double* out,
                                                        double* t, long long s, long long r, long long n, long long s1,
                                                        long long r1) {
	GemmChain ch;
	ch.ns = 2;
	Gemm<double>& v1 = ch.g[0];  // S1((a2,i),c1) = sum_c2 x((a2,i),c2) Rb(c1,c2)
	v1.M = int(r * n); v1.N = int(s1); v1.K = int(r1);
	v1.A = x; v1.sAm = r1; v1.sAk = 1;
	v1.B = Rb; v1.sBk = 1; v1.sBn = r1;
	v1.C = t; v1.sCm = s1; v1.sCn = 1;
	v1.lens(r * n * r1, s1 * r1, r * n * s1);
	Gemm<double>& v2 = ch.g[1];  // Rb'(a1,a2) = sum_(i,c1) b(a1,(i,c1)) S1(a2,(i,c1))
	v2.M = int(s); v2.N = int(r); v2.K = int(n * s1);
	v2.A = bc; v2.sAm = n * s1; v2.sAk = 1;
	v2.B = t; v2.sBk = 1; v2.sBn = n * s1;
	v2.C = out; v2.sCm = r; v2.sCn = 1;
	v2.lens(s * n * s1, r * n * s1, s * r);
	return ch;
}

// One-site local right-hand side b_loc(a,i,b) = sum Lb(s0,a) b_k(s0,i,s1) Rb(s1,b)
// (als.cpp:404-423); scratch t: ra n s1
__host__ __device__ inline GemmChain plan_local_rhs1(const double* Lb, const double* bk, const double* Rb, double* out,
                                                    double* t, long long ra, long long rb, long long s0, long long s1,
                                                    long long n) {
	GemmChain ch;
	ch.ns = 2;
	Gemm<double>& w1 = ch.g[0];
	w1.M = int(ra); w1.N = int(n * s1); w1.K = int(s0);
	w1.A = Lb; w1.sAm = 1; w1.sAk = ra;
	w1.B = bk; w1.sBk = n * s1; w1.sBn = 1;
	w1.C = t; w1.sCm = n * s1; w1.sCn = 1;
	w1.lens(s0 * ra, s0 * n * s1, ra * n * s1);
	Gemm<double>& w3 = ch.g[1];
	w3.M = int(ra * n); w3.N = int(rb); w3.K = int(s1);
	w3.A = t; w3.sAm = s1; w3.sAk = 1;
	w3.B = Rb; w3.sBk = rb; w3.sBn = 1;
	w3.C = out; w3.sCm = rb; w3.sCn = 1;
	w3.lens(ra * n * s1, s1 * rb, ra * n * rb);
	return ch;
}

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
// Mixed form: *flag (device) becomes 1 when the FP64 target was not reached. FP64
// form with gate != nullptr: the launch does nothing unless *gate != 0.
bool cluster_local_solve(Context& c, const LocalShape& s, const double* L, const double* A1, const double* A2,
                         const double* R, const double* b, double* x, double tol, int max_iter, int precision,
                         int* flag = nullptr, const int* gate = nullptr);

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
	bool assume_spd = true;          // false: least squares through A^T A and A^T b (ALS, DMRG, ASD)
	bool use_residual = false;       // useResidualForEndCriterion (als.h:116)
};

struct AlsReport {
	double energy = 0, residual = -1;
	int64_t half_sweeps = 0, micro_steps = 0, local_iterations = 0, refinements = 0;
	std::vector<double> residuals, energies;
	std::vector<int64_t> flags;
};

// A null: the operator-free form, x minimises ||x - b|| (one site only).
AlsReport als(const Tensor* A, Tensor& x, const Tensor& b, const AlsOptions& o);

// Batched one-site ALS_SPD over independent instances in one persistent launch
// (batch.cu). x[i] is updated in place; each x[i] must have maximal-reduced ranks.
struct BatchResult {
	std::vector<double> energy;
	std::vector<int> iterations;
	std::vector<int> final_pos;
	double ms = 0;        // device time of the batch launch (CUDA events)
	int threads = 0, ctas_per_sm = 0, ctas = 0, tile = 0;
};
BatchResult als_batch(Context& c, const std::vector<const Tensor*>& A, const std::vector<Tensor*>& x,
                      const std::vector<const Tensor*>& b, const AlsOptions& o, bool autotune);

// J(x) = <x,Ax> - 2<x,b> and dJ/dX_k for every core.
double als_energy_gradient(const Tensor& A, const Tensor& x, const Tensor& b, std::vector<double>& grad);

}  // namespace xtt
