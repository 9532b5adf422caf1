// Riemannian conjugate gradients on the manifold of TT tensors of fixed rank:
// GeometricCGVariant (src/xerus/algorithms/cg.cpp:34-120) with the submanifold
// retraction and the projective vector transport (src/xerus/algorithms/
// retractions.cpp), and its line search (src/xerus/algorithms/steepestDescent.cpp:37-80).
//
// A tangent vector at a base x (canonical at core 0) is a list of cores V_k shaped like
// x's cores (TTTangentVector). The projection of a TT direction D onto the tangent space
// contracts left stacks <x, D> and <x, x> (the latter pseudo-inverted), a right stack
// <x, D>, and removes from V_k (k > 0) its component along x_k (the gauge condition).
// Every contraction is a small GEMM chain on the device; the algorithm's scalars (step
// lengths, norms, the line search's comparisons) are the host's, as in the reference.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <memory>
#include <vector>

#include "als.cuh"

namespace xtt {

namespace {

__global__ void k_axpy(double* y, const double* x, double f, long long n) {
	for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
		y[i] = fma(f, x[i], y[i]);
}

__global__ void k_scaled_copy(double* y, const double* x, double f, long long n) {
	for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
		y[i] = f * x[i];
}

__global__ void k_reciprocal(double* y, const double* x, int n) {
	for (int i = threadIdx.x; i < n; i += blockDim.x) y[i] = 1.0 / x[i];
}

// A^T core by core: out[k][j][i][l] = A[k][i][j][l]
__global__ void k_op_transpose(double* out, const double* A, int K, int n, int L) {
	const long long total = (long long)K * n * n * L;
	for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
		long long t = e;
		const int l = int(t % L); t /= L;
		const int j = int(t % n); t /= n;
		const int i = int(t % n);
		const int k = int(t / n);
		out[e] = A[((size_t(k) * n + j) * n + i) * L + l];
	}
}

// One core of the TT of a tangent vector (TTTangentVector::operator TTTensor /
// added_to_base, retractions.cpp:163-219): first [U | V] (or [U | U + V]), middle
// [[U, V], [0, U]], last [[V], [U]].
__global__ void k_tangent_block(double* out, const double* U, const double* V, int r0, int n, int r1, int where,
                                int plus_base) {
	const int R0 = where == 0 ? 1 : 2 * r0, R1 = where == 2 ? 1 : 2 * r1;
	const long long total = (long long)R0 * n * R1;
	for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
		const int o1 = int(e % R1), i = int((e / R1) % n), o0 = int(e / ((long long)R1 * n));
		double v = 0.0;
		if (where == 0) {
			const int c = o1 % r1, hi = o1 / r1;
			const double u = U[size_t(i) * r1 + c];
			v = hi == 0 ? u : (plus_base ? u + V[size_t(i) * r1 + c] : V[size_t(i) * r1 + c]);
		} else if (where == 1) {
			const int a = o0 % r0, c = o1 % r1, ha = o0 / r0, hc = o1 / r1;
			const size_t at = (size_t(a) * n + i) * r1 + c;
			v = (ha == hc) ? U[at] : (ha == 0 && hc == 1 ? V[at] : 0.0);
		} else {
			const int a = o0 % r0, ha = o0 / r0;
			v = ha == 0 ? V[size_t(a) * n + i] : U[size_t(a) * n + i];
		}
		out[e] = v;
	}
}

double read_dbl(Context& c, int slot) {
	XTT_CUDA(cudaMemcpyAsync(c.h_dbl + slot, c.d_dbl + slot, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
	c.sync();
	return c.h_dbl[slot];
}

unsigned grid_of(long long n) { return unsigned(std::max<long long>(1, std::min<long long>((n + 255) / 256, 1024))); }

struct DBuf {
	double* p = nullptr;
	DBuf() = default;
	explicit DBuf(size_t n) {
		if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(double)) != cudaSuccess)
			throw Error(XTT_ERR_NO_MEMORY, "device allocation failed (Riemannian CG)");
	}
	DBuf(const DBuf&) = delete;
	DBuf& operator=(const DBuf&) = delete;
	DBuf(DBuf&& o) noexcept : p(o.p) { o.p = nullptr; }
	DBuf& operator=(DBuf&& o) noexcept {
		std::swap(p, o.p);
		return *this;
	}
	~DBuf() {
		if (p) cudaFree(p);
	}
};

void run_chain(Context& c, const GemmChain& ch) {
	for (int i = 0; i < ch.ns; ++i) gemm(c, ch.g[i]);
}

// C (M x N, row-major, ldc) = alpha * op(A) op(B) + beta * C with explicit strides
void mm(Context& c, int M, int N, int K, const double* A, long long sAm, long long sAk, const double* B, long long sBk,
        long long sBn, double* C, long long sCm, long long sCn, double alpha = 1.0, double beta = 0.0) {
	Gemm<double> g;
	g.M = M; g.N = N; g.K = K;
	g.A = A; g.sAm = sAm; g.sAk = sAk;
	g.B = B; g.sBk = sBk; g.sBn = sBn;
	g.C = C; g.sCm = sCm; g.sCn = sCn;
	g.alpha = alpha; g.beta = beta;
	g.lens(Gemm<double>::span(M, 0, sAm, 0) + Gemm<double>::span(K, 0, sAk, 0) + 1,
	       Gemm<double>::span(K, 0, sBk, 0) + Gemm<double>::span(N, 0, sBn, 0) + 1,
	       Gemm<double>::span(M, 0, sCm, 0) + Gemm<double>::span(N, 0, sCn, 0) + 1);
	gemm(c, g);
}

std::unique_ptr<Tensor> clone(const Tensor& x) {
	std::unique_ptr<Tensor> y(new Tensor(x.ctx, x.op, x.d, x.dims.data(), x.ranks.data()));
	y->copy_from(x);
	return y;
}

// pseudo_inverse(M, 1) (src/xerus/tensor.cpp:1568-1574): SVD truncated at EPSILON S[0]
// (calculate_svd's rule), reciprocal singular values; M is r x r, out r x r.
void pseudo_inverse(Context& c, const double* M, int r, double* out) {
	DBuf U(size_t(r) * r), S(r), Vt(size_t(r) * r), Si(r);
	SvdArgs a;
	const size_t wk = svd_work_doubles(r, r);
	DBuf work(wk);
	a.X = M; a.ldx = r; a.m = r; a.n = r; a.max_rank = r; a.eps = 8 * 2.220446049250313e-16;
	a.work = wk ? work.p : nullptr;
	a.U = U.p; a.S = S.p; a.Vt = Vt.p; a.rank_out = c.d_ints + 1; a.status = c.d_status;
	{
		ProfScope ps(c, "svd");
		launch_svd(a, c.stream);
	}
	c.count_launch();
	const int k = c.read_int(1);
	k_reciprocal<<<1, 64, 0, c.stream>>>(Si.p, S.p, k);
	c.count_launch();
	scale_rows(c, Vt.p, Si.p, k, r);  // diag(1/S) Vt
	// out(i, j) = sum_l Vt'(l, i) U(j, l): U is r x min(r, r) row-major
	mm(c, r, r, k, Vt.p, 1, r, U.p, 1, r, out, r, 1);
	XTT_CUDA(cudaGetLastError());
}

struct Tangent {
	std::vector<DBuf> v;  // V_k, shaped like the base's cores
};

// The base (x moved to core 0 with keepRank) and its <x, x> left stacks, shared by the
// projection and the scalar product.
struct Base {
	std::unique_ptr<Tensor> x;
	std::vector<DBuf> uu;  // uu[k]: contraction of cores 0..k-1 with themselves, r_k x r_k
};

Base make_base(const Tensor& x) {
	XTT_REQUIRE(x.canonicalized && x.core_position == 0,
	            "projection onto tangent plane is only implemented for core position 0 at the moment");
	Context& c = *x.ctx;
	Base B;
	B.x = clone(x);
	move_core(*B.x, 0, true);
	const Tensor& U = *B.x;
	B.uu.emplace_back(1);
	fill(c, B.uu[0].p, 1.0, 1);
	for (int k = 0; k + 1 < U.d; ++k) {
		const long long r = U.ranks[k], n = U.dims[k], r1 = U.ranks[k + 1];
		B.uu.emplace_back(size_t(r1 * r1));
		DBuf t(size_t(r * n * r1));
		run_chain(c, plan_push_left_rhs(B.uu[k].p, U.core[k], U.core[k], B.uu[k + 1].p, t.p, r, r, n, r1, r1));
	}
	return B;
}

// TTTangentVector(base, direction) (retractions.cpp:57-103)
Tangent project(Context& c, const Base& B, const Tensor& D) {
	const Tensor& U = *B.x;
	const int d = U.d;
	XTT_REQUIRE(D.d == d && D.dims == U.dims && !D.op, "direction and base dimensions differ");
	std::vector<DBuf> uv;
	uv.emplace_back(1);
	fill(c, uv[0].p, 1.0, 1);
	for (int k = 0; k + 1 < d; ++k) {
		const long long r = U.ranks[k], s = D.ranks[k], n = U.dims[k], r1 = U.ranks[k + 1], s1 = D.ranks[k + 1];
		uv.emplace_back(size_t(r1 * s1));
		DBuf t(size_t(s * n * r1));
		run_chain(c, plan_push_left_rhs(uv[k].p, U.core[k], D.core[k], uv[k + 1].p, t.p, r, s, n, r1, s1));
	}
	Tangent out;
	out.v.resize(d);
	DBuf right(1);
	fill(c, right.p, 1.0, 1);
	for (int k = d - 1; k >= 0; --k) {
		const long long r = U.ranks[k], s = D.ranks[k], n = U.dims[k], r1 = U.ranks[k + 1], s1 = D.ranks[k + 1];
		DBuf inv(size_t(r * r)), t1(size_t(r * s)), t2(size_t(r * n * s1));
		pseudo_inverse(c, B.uu[k].p, int(r), inv.p);
		mm(c, int(r), int(s), int(r), inv.p, r, 1, uv[k].p, s, 1, t1.p, s, 1);                      // inv UV
		mm(c, int(r), int(n * s1), int(s), t1.p, s, 1, D.core[k], n * s1, 1, t2.p, n * s1, 1);    // . D_k
		DBuf V(size_t(r * n * r1));
		mm(c, int(r * n), int(r1), int(s1), t2.p, s1, 1, right.p, 1, s1, V.p, r1, 1);             // . right^T
		if (k != 0) {
			// V -= (V U_k^T) U_k  (the gauge condition)
			DBuf utv(size_t(r * r));
			mm(c, int(r), int(r), int(n * r1), V.p, n * r1, 1, U.core[k], 1, n * r1, utv.p, r, 1);
			mm(c, int(r), int(n * r1), int(r), utv.p, r, 1, U.core[k], n * r1, 1, V.p, n * r1, 1, -1.0, 1.0);
			DBuf nr(size_t(r * s)), t(size_t(s * n * r1));
			run_chain(c, plan_push_right_rhs(right.p, U.core[k], D.core[k], nr.p, t.p, r, s, n, r1, s1));
			right = std::move(nr);
		}
		out.v[k] = std::move(V);
	}
	return out;
}

double tangent_dot(Context& c, const Base& B, const Tangent& a, const Tangent& b) {
	// TTTangentVector::scalar_product (retractions.cpp:143-155)
	const Tensor& U = *B.x;
	double total = 0;
	for (int k = 0; k < U.d; ++k) {
		const long long r = U.ranks[k], n = U.dims[k], r1 = U.ranks[k + 1];
		DBuf t(size_t(r * n * r1));
		mm(c, int(r), int(n * r1), int(r), B.uu[k].p, r, 1, b.v[k].p, n * r1, 1, t.p, n * r1, 1);  // left b
		dot_async(c, a.v[k].p, t.p, size_t(r * n * r1), 40);
		total += read_dbl(c, 40);
	}
	return total;
}

Tangent tangent_combine(Context& c, const Base& B, const Tangent& a, double fa, const Tangent* b, double fb) {
	const Tensor& U = *B.x;
	Tangent out;
	for (int k = 0; k < U.d; ++k) {
		const long long len = (long long)U.core_size(k);
		out.v.emplace_back(size_t(len));
		k_scaled_copy<<<grid_of(len), 256, 0, c.stream>>>(out.v[k].p, a.v[k].p, fa, len);
		c.count_launch();
		if (b) {
			k_axpy<<<grid_of(len), 256, 0, c.stream>>>(out.v[k].p, b->v[k].p, fb, len);
			c.count_launch();
		}
	}
	XTT_CUDA(cudaGetLastError());
	return out;
}

// the TT of a tangent vector (plus_base: added_to_base), canonicalised at 0 (rank-revealing)
std::unique_ptr<Tensor> tangent_tt(Context& c, const Base& B, const Tangent& t, bool plus_base) {
	const Tensor& U = *B.x;
	const int d = U.d;
	std::vector<int64_t> rr(d + 1, 1);
	for (int k = 1; k < d; ++k) rr[k] = 2 * U.ranks[k];
	std::unique_ptr<Tensor> y(new Tensor(&c, false, d, U.dims.data(), rr.data()));
	if (d == 1) {
		k_scaled_copy<<<grid_of(U.core_size(0)), 256, 0, c.stream>>>(y->core[0], t.v[0].p, 1.0, U.core_size(0));
		c.count_launch();
		if (plus_base) {
			k_axpy<<<grid_of(U.core_size(0)), 256, 0, c.stream>>>(y->core[0], U.core[0], 1.0, U.core_size(0));
			c.count_launch();
		}
		y->canonicalized = true;
		y->core_position = 0;
		return y;
	}
	for (int k = 0; k < d; ++k) {
		const int where = k == 0 ? 0 : (k + 1 < d ? 1 : 2);
		k_tangent_block<<<grid_of(y->core_size(k)), 256, 0, c.stream>>>(y->core[k], U.core[k], t.v[k].p, int(U.ranks[k]),
		                                                                 int(U.dims[k]), int(U.ranks[k + 1]), where,
		                                                                 plus_base ? 1 : 0);
		c.count_launch();
	}
	XTT_CUDA(cudaGetLastError());
	y->canonicalized = false;
	move_core(*y, 0, false);
	return y;
}

// SubmanifoldRetractionI (retractions.cpp:228-236): x_k += f V_k, then move_core(0, keepRank)
void retract(Context& c, Tensor& x, const Tangent& t, double f) {
	for (int k = 0; k < x.d; ++k) {
		const long long len = (long long)x.core_size(k);
		k_axpy<<<grid_of(len), 256, 0, c.stream>>>(x.core[k], t.v[k].p, f, len);
		c.count_launch();
	}
	XTT_CUDA(cudaGetLastError());
	x.canonicalized = x.d == 1;
	x.core_position = 0;
	move_core(x, 0, true);
}

// The other retractions of retractions.cpp, for both kinds of step: from the
// point y = x + step (a TT of larger rank: the tangent vector added to its base for
// type I, x + f y for type II) back to x's ranks.
//   HOSVD (HOSVDRetractionI / II, retractions.cpp:43-55): y.round(oldRanks).
//   ALS (ALSRetractionI / II, retractions.cpp:57-69): ALSVariant(1, 2, lapack_solver,
//   false) without an operator, x (the current point, its ranks kept) fitted to y.
void retract_to_ranks(Context& c, Tensor& x, std::unique_ptr<Tensor> y, int kind) {
	(void)c;
	const std::vector<int64_t> old(x.ranks.begin() + 1, x.ranks.end() - 1);
	if (kind == XTT_RETRACTION_HOSVD) {
		round_tt(*y, old, kXerusEpsilon, nullptr);
		x.copy_from(*y);
		return;
	}
	AlsOptions o;
	o.sites = 1;
	o.num_half_sweeps = 2;
	o.convergence_epsilon = 1e-6;
	o.preserve_core_position = true;
	o.assume_spd = false;
	als(nullptr, x, *y, o);
}

// Type I retraction of x (at the tangent's base) along f t.
void retract_i(Context& c, Tensor& x, const Base& B, const Tangent& t, double f, int kind) {
	if (kind == XTT_RETRACTION_SUBMANIFOLD) {
		retract(c, x, t, f);
		return;
	}
	const Tangent ft = tangent_combine(c, B, t, f, nullptr, 0.0);
	retract_to_ranks(c, x, tangent_tt(c, B, ft, true), kind);
}

}  // namespace

RiemannReport geometric_cg(const Tensor* A, Tensor& x, const Tensor& b, int64_t num_steps, double eps, bool assume_spd,
                           int retraction) {
	// GeometricCGVariant::solve (src/xerus/algorithms/cg.cpp:34-120)
	Context& c = *x.ctx;
	XTT_REQUIRE(!x.op && !b.op && x.dims == b.dims && (!A || (A->op && A->dims == x.dims)),
	            "dimensions of A, x and b must match");
	const int d = x.d;
	RiemannReport rep;
	// A^T for the least-squares gradient A^T (b - A x)
	std::unique_ptr<Tensor> At;
	if (A && !assume_spd) {
		At.reset(new Tensor(&c, true, d, A->dims.data(), A->ranks.data()));
		for (int k = 0; k < d; ++k) {
			k_op_transpose<<<grid_of(A->core_size(k)), 256, 0, c.stream>>>(At->core[k], A->core[k], int(A->ranks[k]),
			                                                                int(A->dims[k]), int(A->ranks[k + 1]));
			c.count_launch();
		}
		XTT_CUDA(cudaGetLastError());
	}
	const double norm_b = [&] {
		std::unique_ptr<Tensor> t = clone(b);
		return orthogonal_norm(*t);
	}();
	std::unique_ptr<Tensor> residual;
	// residual = b - A x (b - x without an operator), canonicalised like the reference's sum
	auto calc_residual = [&]() -> double {
		std::unique_ptr<Tensor> ax;
		if (A) {
			std::vector<int64_t> r(d + 1);
			for (int k = 0; k <= d; ++k) r[k] = A->ranks[k] * x.ranks[k];
			ax.reset(new Tensor(&c, false, d, x.dims.data(), r.data()));
			tt_apply(*A, x, *ax);
		} else {
			ax = clone(x);
		}
		residual = clone(b);
		tt_add(*residual, *ax, -1.0);
		std::unique_ptr<Tensor> t = clone(*residual);
		return orthogonal_norm(*t);
	};
	Base base;
	Tangent grad;
	double gnorm = 0;
	auto update_gradient = [&]() {
		base = make_base(x);
		if (At) {
			std::vector<int64_t> r(d + 1);
			for (int k = 0; k <= d; ++k) r[k] = At->ranks[k] * residual->ranks[k];
			Tensor g(&c, false, d, x.dims.data(), r.data());
			tt_apply(*At, *residual, g);
			grad = project(c, base, g);
		} else {
			grad = project(c, base, *residual);
		}
		gnorm = std::sqrt(tangent_dot(c, base, grad, grad));
	};
	double curr = calc_residual();
	const double last = 1e100;  // never updated in the reference's loop
	rep.trace.push_back(curr);
	update_gradient();
	Tangent direction = tangent_combine(c, base, grad, 1.0, nullptr, 0.0);
	double alpha = 1.0;
	int64_t steps = 0;
	while ((num_steps == 0 || steps < num_steps) && curr / norm_b > eps && std::fabs(last - curr) / norm_b > eps &&
	       std::fabs(1.0 - curr / last) / norm_b > eps) {
		++steps;
		const double dir_norm0 = std::sqrt(tangent_dot(c, base, direction, direction));
		double derivative = tangent_dot(c, base, grad, direction) / dir_norm0;
		if (derivative <= 0) {
			direction = tangent_combine(c, base, grad, 1.0, nullptr, 0.0);
			derivative = gnorm;
			alpha = 1.0;
		}
		// line_search (steepestDescent.cpp:37-80), change factor 0.8
		{
			const double change = 0.8;
			const double dir_norm = std::sqrt(tangent_dot(c, base, direction, direction));
			double ca = alpha / change;
			std::unique_ptr<Tensor> old = clone(x);
			retract_i(c, x, base, direction, ca / dir_norm, retraction);
			double best_res = calc_residual();
			double best_alpha = ca;
			std::unique_ptr<Tensor> best = clone(x);
			while (true) {
				ca *= change;
				x.copy_from(*old);
				retract_i(c, x, base, direction, ca / dir_norm, retraction);
				const double r = calc_residual();
				if (r < best_res) {
					best_res = r;
					best_alpha = ca;
					best = clone(x);
				} else {
					break;
				}
			}
			x.copy_from(*best);
			alpha = best_alpha;
			while (alpha > 1e-16 && best_res > curr - 1e-4 * alpha / dir_norm * derivative) {
				alpha *= change;
				x.copy_from(*old);
				retract_i(c, x, base, direction, alpha / dir_norm, retraction);
				best_res = calc_residual();
			}
			curr = best_res;
		}
		// the gradient below uses the residual of the last x the line search evaluated, a
		// rejected trial unless the Armijo loop ran (as in the reference)
		rep.trace.push_back(curr);
		// ProjectiveVectorTransport: the old direction as a TT, projected at the new base
		std::unique_ptr<Tensor> dir_tt = tangent_tt(c, base, direction, false);
		const double old_gnorm = gnorm;
		update_gradient();
		Tangent moved = project(c, base, *dir_tt);
		const double beta = gnorm / old_gnorm;  // Fletcher-Reeves with norms, as in the reference
		direction = tangent_combine(c, base, grad, 1.0, &moved, beta);
	}
	rep.residual = curr;
	rep.steps = steps;
	c.sync();
	return rep;
}

RiemannReport steepest_descent(const Tensor* A, Tensor& x, const Tensor& b, int64_t num_steps, double eps,
                               bool assume_spd, int retraction) {
	// SteepestDescentVariant::solve (src/xerus/algorithms/steepestDescent.cpp:83-175) with
	// SubmanifoldRetractionII (retractions.cpp:222-225), HOSVDRetractionII or ALSRetractionII
	Context& c = *x.ctx;
	XTT_REQUIRE(!x.op && !b.op && x.dims == b.dims && (!A || (A->op && A->dims == x.dims)),
	            "dimensions of A, x and b must match");
	const int d = x.d;
	RiemannReport rep;
	std::unique_ptr<Tensor> At;
	if (A && !assume_spd) {
		At.reset(new Tensor(&c, true, d, A->dims.data(), A->ranks.data()));
		for (int k = 0; k < d; ++k) {
			k_op_transpose<<<grid_of(A->core_size(k)), 256, 0, c.stream>>>(At->core[k], A->core[k], int(A->ranks[k]),
			                                                                int(A->dims[k]), int(A->ranks[k + 1]));
			c.count_launch();
		}
		XTT_CUDA(cudaGetLastError());
	}
	std::unique_ptr<Tensor> residual;
	auto update_residual = [&]() -> double {
		std::unique_ptr<Tensor> ax;
		if (A) {
			std::vector<int64_t> r(d + 1);
			for (int k = 0; k <= d; ++k) r[k] = A->ranks[k] * x.ranks[k];
			ax.reset(new Tensor(&c, false, d, x.dims.data(), r.data()));
			tt_apply(*A, x, *ax);
		} else {
			ax = clone(x);
		}
		residual = clone(b);
		tt_add(*residual, *ax, -1.0);
		std::unique_ptr<Tensor> t = clone(*residual);
		return orthogonal_norm(*t);
	};
	double curr = update_residual(), last = 1e100, alpha = 1.0;
	rep.trace.push_back(curr);
	int64_t steps = 0;
	while ((num_steps == 0 || steps < num_steps) && curr > eps && std::fabs(last - curr) > eps &&
	       std::fabs(1.0 - curr / last) > eps) {
		++steps;
		std::unique_ptr<Tensor> y;
		if (At) {
			std::vector<int64_t> r(d + 1);
			for (int k = 0; k <= d; ++k) r[k] = At->ranks[k] * residual->ranks[k];
			y.reset(new Tensor(&c, false, d, x.dims.data(), r.data()));
			tt_apply(*At, *residual, *y);
		} else {
			y = clone(*residual);
		}
		// the submanifold retraction projects the step at the current x (halving keeps the
		// same base); the others round x + alpha y back to x's ranks
		std::unique_ptr<Tensor> old = clone(x);
		Base base;
		Tangent w;
		if (retraction == XTT_RETRACTION_SUBMANIFOLD) {
			base = make_base(x);
			w = project(c, base, *y);
		}
		auto step = [&](double f) {
			if (retraction == XTT_RETRACTION_SUBMANIFOLD) {
				retract(c, x, w, f);
			} else {
				std::unique_ptr<Tensor> z = clone(x);
				tt_add(*z, *y, f);
				retract_to_ranks(c, x, std::move(z), retraction);
			}
		};
		alpha *= 2;
		step(alpha);
		last = curr;
		curr = update_residual();
		while (alpha > 1e-30 && last < curr) {
			alpha /= 2;
			x.copy_from(*old);
			step(alpha);
			curr = update_residual();
		}
		rep.trace.push_back(curr);
	}
	rep.residual = curr;
	rep.steps = steps;
	c.sync();
	return rep;
}

}  // namespace xtt
