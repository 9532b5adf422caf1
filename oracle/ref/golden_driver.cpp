// Golden-vector driver: runs the xerus reference (linked as libxerus_ref.so)
// on seeded inputs and writes every input and result the parity tests need as
// .npy files into an output directory.
//
//   golden_driver <case> <outdir>
//
// Cases: rng, tt_random, dot, movecore, round, als, dmrg, adf, adf_cfg5, fileio, als_nonspd,
// arith, adf_rankone, gcg, adf_rankinc, qc_gap, retractions, iht, and the timings time_cfg1/2/4/5.
// Every case seeds xerus::misc::randomEngine with 0xBAADF00D and resets
// xerus::misc::defaultNormalDistribution (dropping a cached polar variate) first,
// so a case's draws do not depend on the cases run before it.
#include <xerus.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iterator>
#include <random>
#include <string>
#include <vector>

using namespace xerus;

static std::string g_out;

// ---------------------------------------------------------------- npy output
template <class T> static const char* npy_descr();
template <> const char* npy_descr<double>() { return "<f8"; }
template <> const char* npy_descr<int64_t>() { return "<i8"; }
template <> const char* npy_descr<uint64_t>() { return "<u8"; }
template <> const char* npy_descr<uint8_t>() { return "|u1"; }

template <class T>
static void save(const std::string& name, const std::vector<T>& v, std::vector<size_t> shape = {}) {
	if (shape.empty()) shape = {v.size()};
	std::string dict = std::string("{'descr': '") + npy_descr<T>() + "', 'fortran_order': False, 'shape': (";
	for (size_t i = 0; i < shape.size(); ++i) dict += std::to_string(shape[i]) + (shape.size() == 1 ? "," : (i + 1 < shape.size() ? ", " : ""));
	dict += "), }";
	size_t total = 10 + dict.size() + 1;
	size_t pad = (64 - total % 64) % 64;
	dict += std::string(pad, ' ') + "\n";
	std::ofstream f(g_out + "/" + name + ".npy", std::ios::binary);
	f.write("\x93NUMPY\x01\x00", 8);
	uint16_t hl = uint16_t(dict.size());
	f.write(reinterpret_cast<const char*>(&hl), 2);
	f.write(dict.data(), std::streamsize(dict.size()));
	f.write(reinterpret_cast<const char*>(v.data()), std::streamsize(v.size() * sizeof(T)));
}
static void save_scalar(const std::string& name, double x) { save<double>(name, {x}); }

static void reseed() {
	misc::randomEngine.seed(0xBAADF00D);
	misc::defaultNormalDistribution.reset();
}

// TT layout on disk: <name>_dims (d), <name>_ranks (d+1, boundary ranks 1),
// <name>_cores (all cores concatenated, each row-major (r_{k-1}, n_k, r_k)).
static void save_tt(const std::string& name, const TTTensor& x) {
	const size_t d = x.degree();
	std::vector<int64_t> dims, ranks{1};
	std::vector<double> data;
	for (size_t k = 0; k < d; ++k) {
		Tensor c = x.get_component(k);
		c.use_dense_representation();
		dims.push_back(int64_t(c.dimensions[1]));
		ranks.push_back(int64_t(c.dimensions[2]));
		const double* p = c.get_unsanitized_dense_data();
		for (size_t i = 0; i < c.size; ++i) data.push_back(p[i] * c.factor);
	}
	save(name + "_dims", dims);
	save(name + "_ranks", ranks);
	save(name + "_cores", data);
}

static void save_op(const std::string& name, const TTOperator& A) {
	const size_t d = A.degree() / 2;
	std::vector<int64_t> dims, ranks{1};
	std::vector<double> data;
	for (size_t k = 0; k < d; ++k) {
		Tensor c = A.get_component(k);
		c.use_dense_representation();
		dims.push_back(int64_t(c.dimensions[1]));
		ranks.push_back(int64_t(c.dimensions[3]));
		const double* p = c.get_unsanitized_dense_data();
		for (size_t i = 0; i < c.size; ++i) data.push_back(p[i] * c.factor);
	}
	save(name + "_dims", dims);
	save(name + "_ranks", ranks);
	save(name + "_cores", data);
}

// Entry of a TT at one multi-index, by multiplying the core slices left to right.
static double tt_entry(const TTTensor& x, const std::vector<size_t>& idx) {
	std::vector<double> v{1.0};
	for (size_t k = 0; k < x.degree(); ++k) {
		Tensor c = x.get_component(k);
		c.use_dense_representation();
		const size_t r0 = c.dimensions[0], n = c.dimensions[1], r1 = c.dimensions[2];
		const double* p = c.get_unsanitized_dense_data();
		std::vector<double> w(r1, 0.0);
		for (size_t a = 0; a < r0; ++a)
			for (size_t b = 0; b < r1; ++b) w[b] += v[a] * p[(a * n + idx[k]) * r1 + b] * c.factor;
		v.swap(w);
	}
	return v[0];
}

// Probe positions from a private engine so xerus's own stream is untouched.
static std::vector<std::vector<size_t>> probe_positions(const std::vector<size_t>& dims, size_t count, uint64_t seed) {
	std::mt19937_64 rng(seed);
	std::vector<std::vector<size_t>> out(count, std::vector<size_t>(dims.size()));
	for (auto& p : out)
		for (size_t k = 0; k < dims.size(); ++k) p[k] = size_t(rng() % dims[k]);
	return out;
}

static void save_probes(const std::string& name, const TTTensor& x, const std::vector<std::vector<size_t>>& pos) {
	std::vector<double> vals;
	std::vector<int64_t> flat;
	for (auto& p : pos) {
		vals.push_back(tt_entry(x, p));
		for (auto i : p) flat.push_back(int64_t(i));
	}
	save(name + "_probe_pos", flat, {pos.size(), x.degree()});
	save(name + "_probe_val", vals);
}

static std::vector<int64_t> ranks_of(const TTTensor& x) {
	std::vector<int64_t> r{1};
	for (auto v : x.ranks()) r.push_back(int64_t(v));
	r.push_back(1);
	return r;
}

// 1D Laplacian-sum operator sum_i I x..x (L + V_i) x..x I as a TT operator.
// rank 2: cores [[L+V, I]], [[I,0],[L+V_k,I]], [[I],[L+V]]; V = nullptr means no potential.
// rank 3 (potential carried in its own channel): [[L+V_0, I, I]], [[I,0,0],[L,I,0],[V_k,0,I]], [[I],[L],[V]].
static TTOperator laplace_operator(size_t d, size_t n, const std::vector<std::vector<double>>* V, bool rank3, double shift = 0.0,
                                   double convection = 0.0) {
	TTOperator A(std::vector<size_t>(2 * d, n));
	// tridiag(-1, 2, -1), plus convection * tridiag(-1, 0, 1) (not symmetric when convection != 0)
	auto L = [&](size_t i, size_t j) {
		return (i == j ? 2.0 : 0.0) - ((i + 1 == j || j + 1 == i) ? 1.0 : 0.0) +
		       convection * ((i + 1 == j ? 1.0 : 0.0) - (j + 1 == i ? 1.0 : 0.0));
	};
	auto I = [&](size_t i, size_t j) { return i == j ? 1.0 : 0.0; };
	auto Vd = [&](size_t k, size_t i, size_t j) { return (V && i == j) ? (*V)[k][i] : 0.0; };
	const size_t R = rank3 ? 3 : 2;
	for (size_t k = 0; k < d; ++k) {
		const size_t rl = k == 0 ? 1 : R, rr = k + 1 == d ? 1 : R;
		Tensor c({rl, n, n, rr}, Tensor::Representation::Dense);
		for (size_t i = 0; i < n; ++i)
			for (size_t j = 0; j < n; ++j) {
				const double l = L(i, j) + (rank3 ? 0.0 : Vd(k, i, j)) + shift * I(i, j) / double(d);
				auto at = [&](size_t a, size_t b) -> double& { return c[((a * n + i) * n + j) * rr + b]; };
				if (d == 1) { at(0, 0) = L(i, j) + Vd(k, i, j) + shift * I(i, j); continue; }
				if (k == 0) {
					at(0, 0) = l + (rank3 ? Vd(k, i, j) : 0.0);
					at(0, 1) = I(i, j);
					if (rank3) at(0, 2) = I(i, j);
				} else if (k + 1 == d) {
					at(0, 0) = I(i, j);
					at(1, 0) = l;
					if (rank3) at(2, 0) = Vd(k, i, j);
				} else {
					at(0, 0) = I(i, j);
					at(1, 0) = l;
					at(1, 1) = I(i, j);
					if (rank3) { at(2, 0) = Vd(k, i, j); at(2, 2) = I(i, j); }
				}
			}
		A.set_component(k, c);
	}
	return A;
}

// x (+) c*x as a non-canonical TT with every inner rank doubled: the same tensor
// (1+c)*x in a rank-deficient representation, built core by core.
static TTTensor block_sum(const TTTensor& x, double c) {
	const size_t d = x.degree();
	TTTensor z(x.dimensions);
	for (size_t k = 0; k < d; ++k) {
		Tensor a = x.get_component(k);
		a.use_dense_representation();
		const size_t r0 = a.dimensions[0], n = a.dimensions[1], r1 = a.dimensions[2];
		const size_t R0 = k == 0 ? 1 : 2 * r0, R1 = k + 1 == d ? 1 : 2 * r1;
		Tensor b({R0, n, R1}, Tensor::Representation::Dense);
		for (size_t i = 0; i < r0; ++i)
			for (size_t j = 0; j < n; ++j)
				for (size_t l = 0; l < r1; ++l) {
					const double v = a[(i * n + j) * r1 + l];
					b[(i * n + j) * R1 + l] = v;
					const size_t i2 = k == 0 ? i : r0 + i, l2 = k + 1 == d ? l : r1 + l;
					b[(i2 * n + j) * R1 + l2] += (k == 0 ? c : 1.0) * v;
				}
		z.set_component(k, b);
	}
	return z;
}

// ||A x - b|| / ||b|| through full (dense) tensors: only for small total sizes.
static double dense_residual(const TTOperator& A, const TTTensor& x, const TTTensor& b) {
	Index i, j;
	TTTensor Ax;
	Ax(i & 0) = A(i / 2, j / 2) * x(j & 0);
	Tensor fa(Ax), fb(b);
	double s = 0, nb = 0;
	for (size_t t = 0; t < fa.size; ++t) { s += (fa[t] - fb[t]) * (fa[t] - fb[t]); nb += fb[t] * fb[t]; }
	return std::sqrt(s / nb);
}

static double residual_of(const TTOperator& A, const TTTensor& x, const TTTensor& b) {
	Index i, j;
	TTTensor Ax;
	Ax(i & 0) = A(i / 2, j / 2) * x(j & 0);
	return frob_norm(Ax - b) / frob_norm(b);
}

static std::vector<double> perf_residuals(const PerformanceData& p, std::vector<int64_t>* flags = nullptr) {
	std::vector<double> r;
	for (auto& dp : p.data) {
		r.push_back(dp.residual);
		if (flags) flags->push_back(int64_t(dp.flags));
	}
	return r;
}

// ------------------------------------------------------------------- cases
static void case_rng() {
	reseed();
	std::vector<uint64_t> raw;
	for (int i = 0; i < 64; ++i) raw.push_back(misc::randomEngine());
	save("rng_raw_u64", raw);
	reseed();
	std::vector<double> normals;
	for (int i = 0; i < 257; ++i) normals.push_back(misc::defaultNormalDistribution(misc::randomEngine));
	save("rng_normal", normals);
	reseed();
	std::vector<double> scaled;
	std::normal_distribution<double> d8(0.0, 0.125);
	for (int i = 0; i < 129; ++i) scaled.push_back(d8(misc::randomEngine));
	save("rng_normal_sd0125", scaled);
	reseed();
	std::vector<int64_t> ints;
	for (size_t n : {2, 3, 4, 5, 7, 8, 10, 1000}) {
		std::uniform_int_distribution<size_t> u(0, n - 1);
		for (int i = 0; i < 32; ++i) ints.push_back(int64_t(u(misc::randomEngine)));
	}
	save("rng_uniform_int", ints);
	reseed();
	std::vector<double> unif;
	std::uniform_real_distribution<double> ur(0.0, 1.0);
	for (int i = 0; i < 64; ++i) unif.push_back(ur(misc::randomEngine));
	save("rng_uniform_real", unif);
}

static void case_tt_random() {
	// A small TT whose ranks get clipped by the dimensions, returned by random() after move_core(0).
	reseed();
	TTTensor x = TTTensor::random({3, 4, 2, 5}, {2, 7, 3});
	save_tt("small", x);
	Tensor full(x);
	std::vector<double> f(full.size);
	for (size_t i = 0; i < full.size; ++i) f[i] = full[i];
	save("small_full", f);
	save_scalar("small_norm", frob_norm(x));
	std::vector<int64_t> r = ranks_of(x);
	save("small_ranks_after", r);
	// cfg1-size TT (d=8, n=4, rank 8) for entry-level comparison.
	reseed();
	TTTensor y = TTTensor::random(std::vector<size_t>(8, 4), 8);
	save_tt("d8", y);
	auto pos = probe_positions(std::vector<size_t>(8, 4), 200, 7);
	save_probes("d8", y, pos);
	save_scalar("d8_norm", frob_norm(y));
}

static void case_dot() {
	// Two independent d=32, n=4, rank-64 TTs with entries N(0, 1/8) (std-dev 1/sqrt(64)).
	reseed();
	std::normal_distribution<double> dist(0.0, 0.125);
	const std::vector<size_t> dims(32, 4);
	TTTensor x = TTTensor::random(dims, std::vector<size_t>(31, 64), dist, misc::randomEngine);
	TTTensor y = TTTensor::random(dims, std::vector<size_t>(31, 64), dist, misc::randomEngine);
	Index i;
	const double xy = value_t(x(i & 0) * y(i & 0));
	const double xx = value_t(x(i & 0) * x(i & 0));
	save_scalar("cfg2_dot_xy", xy);
	save_scalar("cfg2_dot_xx", xx);
	save_scalar("cfg2_norm_x", frob_norm(x));
	save_scalar("cfg2_norm_y", frob_norm(y));
	save("cfg2_ranks_x", ranks_of(x));
	auto pos = probe_positions(dims, 64, 11);
	save_probes("cfg2_x", x, pos);
	save_probes("cfg2_y", y, pos);
	// Small, non-canonical pair: full contraction path, no core shortcut.
	reseed();
	TTTensor a = TTTensor::random({2, 3, 4, 3, 2}, {2, 3, 3, 2});
	TTTensor b = TTTensor::random({2, 3, 4, 3, 2}, {1, 4, 2, 2});
	save_tt("small_a", a);
	save_tt("small_b", b);
	save_scalar("small_dot", value_t(a(i & 0) * b(i & 0)));
	TTTensor s = a + b;  // rank-summed, not canonicalized
	save_scalar("small_sum_norm", frob_norm(s));
}

static void case_movecore() {
	reseed();
	TTTensor x = TTTensor::random({4, 3, 5, 2, 4, 3}, {3, 6, 4, 5, 3});
	save_tt("x", x);
	auto pos = probe_positions({4, 3, 5, 2, 4, 3}, 100, 3);
	for (size_t p : {5, 2, 0, 3}) {
		TTTensor y = x;
		y.move_core(p, true);
		save_probes("qr_to" + std::to_string(p), y, pos);
		save("qr_to" + std::to_string(p) + "_ranks", ranks_of(y));
		save_scalar("qr_to" + std::to_string(p) + "_corenorm", y.get_component(p).frob_norm());
	}
	// Rank-deficient representation: x + 2x has every rank doubled but the
	// same tensor; QC-based move_core may shrink ranks (only when R[0,0] > 0).
	TTTensor z = block_sum(x, 2.0);
	save_tt("z", z);
	save("z_ranks_before", ranks_of(z));
	for (size_t p : {5, 0}) {
		TTTensor y = z;
		y.move_core(p, false);
		save("qc_to" + std::to_string(p) + "_ranks", ranks_of(y));
		save_probes("qc_to" + std::to_string(p), y, pos);
	}
	{
		TTTensor y = z;
		y.canonicalize_left();
		save("z_left_ranks", ranks_of(y));
		y.round(1e-12);
		save("z_round_eps_ranks", ranks_of(y));
		save_probes("z_round_eps", y, pos);
	}
}

// Replays TTNetwork::round(maxRanks, eps) edge by edge through the public
// round_edge, reading the bond singular values after each edge: at that point
// the cores left of the bond are left-orthogonal and those right of it
// right-orthogonal, so the SVD of the absorbing core equals the truncated S.
static std::vector<double> round_with_spectra(TTTensor& x, const std::vector<size_t>& maxRanks, double eps) {
	const size_t d = x.degree();
	std::vector<double> spectra;
	x.canonicalize_right();
	for (size_t i = 0; i + 1 < d; ++i) {
		x.round_edge(d - i, d - i - 1, maxRanks[d - i - 2], eps, 0.0);
		const Tensor& to = x.get_component(d - i - 2);
		Tensor U, S, Vt;
		calculate_svd(U, S, Vt, to, 2, 0, 0.0);
		const size_t r = S.dimensions[0];
		for (size_t j = 0; j < r; ++j) spectra.push_back(S[j * r + j]);
	}
	x.assume_core_position(0);
	return spectra;
}

static void case_round() {
	reseed();
	std::normal_distribution<double> dist(0.0, 0.125);
	const std::vector<size_t> dims(32, 4);
	TTTensor x = TTTensor::random(dims, std::vector<size_t>(31, 64), dist, misc::randomEngine);
	auto pos = probe_positions(dims, 64, 11);
	TTTensor y = x;
	y.round(size_t(32));
	save("cfg2_round_ranks", ranks_of(y));
	save_scalar("cfg2_round_norm", frob_norm(y));
	Index i;
	save_scalar("cfg2_round_dot_x", value_t(y(i & 0) * x(i & 0)));
	save_probes("cfg2_round", y, pos);
	TTTensor z = x;
	auto spectra = round_with_spectra(z, std::vector<size_t>(31, 32), EPSILON);
	save("cfg2_round_spectra", spectra);
	save("cfg2_round_replay_ranks", ranks_of(z));
	save_probes("cfg2_round_replay", z, pos);
	// Time the reference round on this input (1 thread unless OPENBLAS_NUM_THREADS says otherwise).
	{
		TTTensor w = x;
		auto t0 = std::chrono::steady_clock::now();
		w.round(size_t(32));
		auto t1 = std::chrono::steady_clock::now();
		save_scalar("cfg2_round_seconds", std::chrono::duration<double>(t1 - t0).count());
	}
	// Small eps-driven rounding: a rank-3 TT plus a 1e-9 perturbation of rank 2.
	reseed();
	const std::vector<size_t> sd{3, 4, 3, 4, 3};
	TTTensor a = TTTensor::random(sd, {3, 3, 3, 3});
	TTTensor e = TTTensor::random(sd, {2, 2, 2, 2});
	TTTensor s = a + 1e-9 * e;
	save_tt("eps_in", s);
	auto spos = probe_positions(sd, 100, 5);
	TTTensor s1 = s;
	s1.round(1e-6);
	save("eps_round_ranks", ranks_of(s1));
	save_probes("eps_round", s1, spos);
	TTTensor s2 = s;
	auto sp2 = round_with_spectra(s2, std::vector<size_t>(4, std::numeric_limits<size_t>::max()), 1e-6);
	save("eps_round_spectra", sp2);
	TTTensor s3 = s;
	s3.round(std::vector<size_t>{2, 5, 2, 5}, 0.0);
	save("maxr_round_ranks", ranks_of(s3));
	save_probes("maxr_round", s3, spos);
}

static void run_als(const std::string& tag, const ALSVariant& variant, const TTOperator& A, TTTensor x, const TTTensor& b,
                    size_t halfSweeps, const std::vector<std::vector<size_t>>& pos) {
	PerformanceData perf(false, true);
	const double energy = variant(A, x, b, halfSweeps, perf);
	std::vector<int64_t> flags;
	save(tag + "_perf_residual", perf_residuals(perf, &flags));
	save(tag + "_perf_flags", flags);
	save_scalar(tag + "_energy", energy);
	save_scalar(tag + "_final_residual", residual_of(A, x, b));
	if (x.degree() <= 8) save_scalar(tag + "_dense_residual", dense_residual(A, x, b));
	save(tag + "_ranks", ranks_of(x));
	save_probes(tag + "_x", x, pos);
	save_scalar(tag + "_norm_x", frob_norm(x));
}

static void case_als() {
	// Laplacian-sum on d=8, n=4 (operator rank 2); b random rank 4; x0 random rank 8, normalised.
	reseed();
	const size_t d = 8, n = 4;
	TTOperator A = laplace_operator(d, n, nullptr, false);
	TTTensor b = TTTensor::random(std::vector<size_t>(d, n), 4);
	TTTensor x = TTTensor::random(std::vector<size_t>(d, n), 8);
	x /= frob_norm(x);
	save_op("A", A);
	save_tt("b", b);
	save_tt("x0", x);
	auto pos = probe_positions(std::vector<size_t>(d, n), 200, 13);
	ALSVariant als = ALS_SPD;
	als.convergenceEpsilon = 0.0;
	run_als("r8_hs20", als, A, x, b, 20, pos);
	run_als("r8_hs3", als, A, x, b, 3, pos);
	ALSVariant asd = ASD_SPD;
	asd.convergenceEpsilon = 0.0;
	run_als("r8_asd_hs4", asd, A, x, b, 4, pos);
	// Default variant: stops on |dE| < 1e-6.
	run_als("r8_default", ALS_SPD, A, x, b, 20, pos);
	// Rank 32: reaches the 1e-8 residual target within two half-sweeps.
	reseed();
	TTTensor b2 = TTTensor::random(std::vector<size_t>(d, n), 4);
	TTTensor x2 = TTTensor::random(std::vector<size_t>(d, n), 32);
	x2 /= frob_norm(x2);
	save_tt("x0_r32", x2);
	save_tt("b_r32", b2);
	run_als("r32_hs2", als, A, x2, b2, 2, pos);
	// Ragged: odd dims, ranks clipped by dimensions.
	reseed();
	const std::vector<size_t> rd{3, 5, 2, 4, 3};
	TTOperator A3(std::vector<size_t>(10, 1));
	{
		// Laplacian sum on uneven mode sizes plus a constant shift 0.5 on the first mode.
		TTOperator Ar(std::vector<size_t>{3, 5, 2, 4, 3, 3, 5, 2, 4, 3});
		for (size_t k = 0; k < 5; ++k) {
			const size_t m = rd[k], rl = k == 0 ? 1 : 2, rr = k == 4 ? 1 : 2;
			Tensor c({rl, m, m, rr}, Tensor::Representation::Dense);
			for (size_t i = 0; i < m; ++i)
				for (size_t j = 0; j < m; ++j) {
					double l = (i == j ? 2.0 : 0.0) - ((i + 1 == j || j + 1 == i) ? 1.0 : 0.0) + (k == 0 && i == j ? 0.5 : 0.0);
					double id = i == j ? 1.0 : 0.0;
					auto at = [&](size_t a, size_t b_) -> double& { return c[((a * m + i) * m + j) * rr + b_]; };
					if (k == 0) { at(0, 0) = l; at(0, 1) = id; }
					else if (k == 4) { at(0, 0) = id; at(1, 0) = l; }
					else { at(0, 0) = id; at(1, 0) = l; at(1, 1) = id; }
				}
			Ar.set_component(k, c);
		}
		A3 = Ar;
	}
	TTTensor b3 = TTTensor::random(rd, {2, 3, 3, 2});
	TTTensor x3 = TTTensor::random(rd, {3, 4, 4, 3});
	save_op("A_rag", A3);
	save_tt("b_rag", b3);
	save_tt("x0_rag", x3);
	auto rpos = probe_positions(rd, 100, 17);
	run_als("rag_hs6", als, A3, x3, b3, 6, rpos);
}

// ALSVariant::operator()(x, b, ...) without an operator: minimises ||x - b||.
static void run_approx(const std::string& tag, const ALSVariant& variant, TTTensor x, const TTTensor& b, size_t halfSweeps,
                       const std::vector<std::vector<size_t>>& pos) {
	PerformanceData perf(false, true);
	const double energy = variant(x, b, halfSweeps, perf);
	std::vector<int64_t> flags;
	save(tag + "_perf_residual", perf_residuals(perf, &flags));
	save(tag + "_perf_flags", flags);
	save_scalar(tag + "_energy", energy);
	save_scalar(tag + "_final_distance", frob_norm(x - b));
	save(tag + "_ranks", ranks_of(x));
	save_probes(tag + "_x", x, pos);
}

static void case_als_nonspd() {
	// Non-symmetric operator: sum over modes of L + 0.6 * tridiag(-1, 0, 1) (rank 2), d=6, n=4.
	reseed();
	const size_t d = 6, n = 4;
	const std::vector<size_t> dims(d, n);
	TTOperator A = laplace_operator(d, n, nullptr, false, 0.0, 0.6);
	TTTensor b = TTTensor::random(dims, 3);
	TTTensor x = TTTensor::random(dims, 4);
	x /= frob_norm(x);
	save_op("A", A);
	save_tt("b", b);
	save_tt("x0", x);
	auto pos = probe_positions(dims, 200, 29);
	ALSVariant als = ALS;
	als.convergenceEpsilon = 0.0;
	run_als("als_hs6", als, A, x, b, 6, pos);
	ALSVariant asd = ASD;
	asd.convergenceEpsilon = 0.0;
	run_als("asd_hs6", asd, A, x, b, 6, pos);
	ALSVariant dmrg = DMRG;
	dmrg.convergenceEpsilon = 0.0;
	run_als("dmrg_hs3", dmrg, A, x, b, 3, pos);
	// default variant: stops on |d residual| < 1e-6
	run_als("als_default", ALS, A, x, b, 40, pos);
	// SPD operator with the residual as the end criterion (useResidualForEndCriterion)
	TTOperator As = laplace_operator(d, n, nullptr, false);
	save_op("A_spd", As);
	ALSVariant res = ALS_SPD;
	res.useResidualForEndCriterion = true;
	run_als("spd_useres", res, As, x, b, 20, pos);
	// without an operator: x (rank 3) approximates c (rank 6)
	TTTensor c = TTTensor::random(dims, 6);
	TTTensor y = TTTensor::random(dims, 3);
	save_tt("c", c);
	save_tt("y0", y);
	ALSVariant approx = ALS;
	approx.convergenceEpsilon = 0.0;
	run_approx("free_hs4", approx, y, c, 4, pos);
	ALSVariant approx_res = ALS;
	approx_res.useResidualForEndCriterion = true;
	run_approx("free_useres", approx_res, y, c, 10, pos);
}

static void save_full(const std::string& name, const TTTensor& x) {
	Tensor full(x);
	std::vector<double> f(full.size);
	for (size_t i = 0; i < full.size; ++i) f[i] = full[i];
	save(name + "_full", f);
	save(name + "_ranks", ranks_of(x));
	save<int64_t>(name + "_canon", {int64_t(x.canonicalized), int64_t(x.corePosition)});
}

static void case_arith() {
	// TT sums (operator+=, operator-=) and operator products (TTStack casts), d=5, n=4.
	reseed();
	const size_t d = 5, n = 4;
	const std::vector<size_t> dims(d, n);
	TTTensor x = TTTensor::random(dims, 3);
	TTTensor y = TTTensor::random(dims, 2);
	TTOperator Ar = TTOperator::random(std::vector<size_t>(2 * d, n), 2);
	TTOperator A = laplace_operator(d, n, nullptr, false, 0.0, 0.6);
	save_tt("x", x);
	save_tt("y", y);
	save_op("Ar", Ar);
	save_op("A", A);
	save<int64_t>("Ar_canon", {int64_t(Ar.canonicalized), int64_t(Ar.corePosition)});
	save<int64_t>("A_canon", {int64_t(A.canonicalized), int64_t(A.corePosition)});
	save_full("sum", x + y);
	save_full("diff", x - y);
	save_full("twice", x + x);
	Index i, j, k;
	TTTensor p;
	p(i & 0) = A(i / 2, j / 2) * x(j & 0);
	save_full("Ax", p);
	TTTensor q;
	q(i & 0) = Ar(i / 2, j / 2) * x(j & 0);
	save_full("Arx", q);
	save_full("Ax_plus_x", p + x);
	TTOperator AA;
	AA(i / 2, k / 2) = A(i / 2, j / 2) * Ar(j / 2, k / 2);
	std::vector<int64_t> ar;
	for (size_t r : AA.ranks()) ar.push_back(int64_t(r));
	save("AAr_ranks", ar);
	save<int64_t>("AAr_canon", {int64_t(AA.canonicalized), int64_t(AA.corePosition)});
	TTTensor w;
	w(i & 0) = AA(i / 2, j / 2) * x(j & 0);
	save_full("AAr_x", w);
}

// Riemannian CG on the fixed-rank TT manifold (GeometricCGVariant, algorithms/cg.cpp) with
// SubmanifoldRetractionI and ProjectiveVectorTransport (algorithms/retractions.cpp).
static void run_gcg(const std::string& tag, const GeometricCGVariant& v, const TTOperator* A, TTTensor x,
                    const TTTensor& b, size_t steps, const std::vector<std::vector<size_t>>& pos) {
	PerformanceData perf(false, true);
	const double res = A ? v(*A, x, b, steps, perf) : v(x, b, steps, perf);
	save(tag + "_perf_residual", perf_residuals(perf));
	save_scalar(tag + "_residual", res);
	save(tag + "_ranks", ranks_of(x));
	save_probes(tag + "_x", x, pos);
	save_tt(tag + "_x", x);
}

static void case_gcg() {
	reseed();
	const size_t d = 5, n = 3;
	const std::vector<size_t> dims(d, n);
	TTOperator A = laplace_operator(d, n, nullptr, false, 1.0);
	TTOperator An = laplace_operator(d, n, nullptr, false, 1.0, 0.4);
	TTTensor b = TTTensor::random(dims, 2);
	TTTensor x = TTTensor::random(dims, 2);
	save_op("A", A);
	save_op("An", An);
	save_tt("b", b);
	save_tt("x0", x);
	auto pos = probe_positions(dims, 100, 37);
	GeometricCGVariant spd = GeometricCG;
	spd.assumeSymmetricPositiveDefiniteOperator = true;
	run_gcg("spd", spd, &A, x, b, 12, pos);
	run_gcg("ls", GeometricCG, &An, x, b, 12, pos);
	run_gcg("free", GeometricCG, nullptr, x, b, 8, pos);
	// steepest descent with the submanifold retraction (algorithms/steepestDescent.cpp)
	auto run_sd = [&](const std::string& tag, const SteepestDescentVariant& v, const TTOperator* Ap, size_t steps) {
		TTTensor y = x;
		PerformanceData perf(false, true);
		const double res = Ap ? v(*Ap, y, b, steps, perf) : v(y, b, steps, perf);
		save(tag + "_perf_residual", perf_residuals(perf));
		save_scalar(tag + "_residual", res);
		save_probes(tag + "_x", y, pos);
	};
	SteepestDescentVariant sds = SteepestDescent;
	sds.assumeSymmetricPositiveDefiniteOperator = true;
	run_sd("sd_spd", sds, &A, 10);
	run_sd("sd_ls", SteepestDescent, &An, 10);
	run_sd("sd_free", SteepestDescent, nullptr, 6);
}

// The HOSVD and ALS retractions (retractions.cpp:43-69) in GeometricCG (type I, with the
// projective vector transport) and SteepestDescent (type II), on the gcg case's inputs.
static void case_retractions() {
	reseed();
	const size_t d = 5, n = 3;
	const std::vector<size_t> dims(d, n);
	TTOperator A = laplace_operator(d, n, nullptr, false, 1.0);
	TTOperator An = laplace_operator(d, n, nullptr, false, 1.0, 0.4);
	TTTensor b = TTTensor::random(dims, 2);
	TTTensor x = TTTensor::random(dims, 2);
	save_op("A", A);
	save_op("An", An);
	save_tt("b", b);
	save_tt("x0", x);
	auto pos = probe_positions(dims, 100, 47);
	const std::vector<std::pair<std::string, TTRetractionI>> r1{{"hosvd", HOSVDRetractionI}, {"als", ALSRetractionI}};
	for (const auto& r : r1) {
		run_gcg("gcg_" + r.first + "_spd", GeometricCGVariant(0, 1e-8, true, r.second, ProjectiveVectorTransport), &A, x,
		        b, 8, pos);
		run_gcg("gcg_" + r.first + "_ls", GeometricCGVariant(0, 1e-8, false, r.second, ProjectiveVectorTransport), &An,
		        x, b, 8, pos);
	}
	const std::vector<std::pair<std::string, TTRetractionII>> r2{{"hosvd", HOSVDRetractionII}, {"als", ALSRetractionII}};
	for (const auto& r : r2) {
		for (int spd = 1; spd >= 0; --spd) {
			TTTensor y = x;
			PerformanceData perf(false, true);
			SteepestDescentVariant v(0, 1e-8, spd != 0, r.second);
			const double res = v(spd ? A : An, y, b, size_t(8), perf);
			const std::string tag = "sd_" + r.first + (spd ? "_spd" : "_ls");
			save(tag + "_perf_residual", perf_residuals(perf));
			save_scalar(tag + "_residual", res);
			save(tag + "_ranks", ranks_of(y));
			save_probes(tag + "_x", y, pos);
		}
	}
}

static void case_dmrg() {
	reseed();
	const size_t d = 8, n = 4;
	TTOperator A = laplace_operator(d, n, nullptr, false);
	TTTensor b = TTTensor::random(std::vector<size_t>(d, n), 4);
	TTTensor x = TTTensor::random(std::vector<size_t>(d, n), 4);
	x /= frob_norm(x);
	save_op("A", A);
	save_tt("b", b);
	save_tt("x0", x);
	auto pos = probe_positions(std::vector<size_t>(d, n), 200, 19);
	ALSVariant dmrg = DMRG_SPD;
	dmrg.convergenceEpsilon = 0.0;
	run_als("d8_r4_hs4", dmrg, A, x, b, 4, pos);
	// Laplacian plus a per-mode diagonal potential U[0,1], rank-3 operator, d=20, n=8, x rank 8.
	// The reference's 2-site local operator only assembles when site 0 is pruned
	// (first rank >= n), so x starts at rank 8 = n here.
	reseed();
	const size_t d3 = 20, n3 = 8;
	std::vector<std::vector<double>> V(d3, std::vector<double>(n3));
	std::uniform_real_distribution<double> u01(0.0, 1.0);
	for (auto& v : V)
		for (auto& e : v) e = u01(misc::randomEngine);
	TTOperator A3 = laplace_operator(d3, n3, &V, true);
	TTTensor b3 = TTTensor::random(std::vector<size_t>(d3, n3), 4);
	TTTensor x3 = TTTensor::random(std::vector<size_t>(d3, n3), 8);
	x3 /= frob_norm(x3);
	save_op("A_pot", A3);
	save_tt("b_pot", b3);
	save_tt("x0_pot", x3);
	auto pos3 = probe_positions(std::vector<size_t>(d3, n3), 200, 23);
	run_als("pot_r8_hs2", dmrg, A3, x3, b3, 2, pos3);
}

// Reaches ADF's protected internals to read the projected gradient of the
// first sweep step, the quantity the adjoint kernel must reproduce.
struct AdfProbe : ADFVariant {
	AdfProbe() : ADFVariant(1, 0.0, 1.0) {}
	struct Solver : InternalSolver<SinglePointMeasurementSet> {
		using Base = InternalSolver<SinglePointMeasurementSet>;
		Solver(TTTensor& x, const SinglePointMeasurementSet& m, PerformanceData& p)
		    : Base(x, x.ranks(), m, 1, 0.0, 1.0, p) {}
		// Projected gradient and slice norms at every core position of the first sweep.
		void run(std::vector<double>& grads, std::vector<double>& slicenorms, std::vector<double>& resid0) {
			construct_stacks(forwardStackSaveSlots, forwardUpdates, forwardStackMem, true);
			construct_stacks(backwardStackSaveSlots, backwardUpdates, backwardStackMem, false);
			x.canonicalize_left();
			resize_stack_tensors();
			x.move_core(0, true);
			for (size_t k = x.degree() - 1; k > 0; --k) update_backward_stack(k, x.get_component(k));
			calculate_residual(0);
			resid0 = residual;
			for (size_t k = 0; k < degree; ++k) {
				if (k > 0) calculate_residual(k);
				calculate_projected_gradient(k);
				const Tensor& g = projectedGradientComponent;
				for (size_t i = 0; i < g.size; ++i) grads.push_back(g[i]);
				auto nrm = calculate_slicewise_norm_A_projGrad(k);
				slicenorms.insert(slicenorms.end(), nrm.begin(), nrm.end());
				update_x(nrm, k);
				if (k + 1 < degree) {
					x.move_core(k + 1, true);
					update_forward_stack(k, x.get_component(k));
				}
			}
		}
	};
};

static void adf_case(const std::string& tag, const std::vector<size_t>& dims, size_t rank, size_t N, size_t iters,
                     bool savePositions, bool probeGradient) {
	reseed();
	TTTensor target = TTTensor::random(dims, rank);
	SinglePointMeasurementSet m = SinglePointMeasurementSet::random(N, dims);
	m.measure(target);
	std::vector<double> clean = m.measuredValues;
	std::normal_distribution<double> noise(0.0, 1e-6);
	for (auto& v : m.measuredValues) v += noise(misc::randomEngine);
	TTTensor x = TTTensor::random(dims, rank);
	save_tt(tag + "_target", target);
	save_tt(tag + "_x0", x);
	const size_t d = dims.size();
	std::vector<uint8_t> pos8;
	std::vector<uint64_t> h{1469598103934665603ull};
	for (auto& p : m.positions)
		for (auto i : p) {
			pos8.push_back(uint8_t(i));
			h[0] = (h[0] ^ uint64_t(i)) * 1099511628211ull;
		}
	save(tag + "_positions_fnv1a", h);
	if (savePositions) {
		save(tag + "_positions", pos8, {N, d});
		save(tag + "_values", m.measuredValues);
	} else {
		std::vector<uint8_t> head(pos8.begin(), pos8.begin() + 64 * d);
		save(tag + "_positions_head", head, {64, d});
		save(tag + "_values_head", std::vector<double>(m.measuredValues.begin(), m.measuredValues.begin() + 64));
	}
	double vsum = 0;
	for (auto v : m.measuredValues) vsum += v;
	save_scalar(tag + "_values_sum", vsum);
	save_scalar(tag + "_clean_sum", [&] { double s = 0; for (auto v : clean) s += v; return s; }());
	if (probeGradient) {
		TTTensor xg = x;
		PerformanceData none(false, false);
		AdfProbe::Solver s(xg, m, none);
		std::vector<double> grads, norms, r0;
		s.run(grads, norms, r0);
		save(tag + "_grad_sweep", grads);
		save(tag + "_slicenorm_sweep", norms);
		if (savePositions) save(tag + "_residual0", r0);
		else save(tag + "_residual0_head", std::vector<double>(r0.begin(), r0.begin() + 64));
		double r0sq = 0;
		for (auto v : r0) r0sq += v * v;
		save_scalar(tag + "_residual0_sqsum", r0sq);
		save_tt(tag + "_x_after_sweep1", xg);
	}
	PerformanceData perf(false, true);
	ADFVariant adf(iters, 0.0, 1.0);
	auto t0 = std::chrono::steady_clock::now();
	const double res = adf(x, m, perf);
	auto t1 = std::chrono::steady_clock::now();
	save_scalar(tag + "_seconds", std::chrono::duration<double>(t1 - t0).count());
	save(tag + "_perf_residual", perf_residuals(perf));
	save_scalar(tag + "_final_residual", res);
	save_tt(tag + "_x_final", x);
	auto pos = probe_positions(dims, 100, 29);
	save_probes(tag + "_x_final", x, pos);
}

static void case_adf() { adf_case("small", {4, 5, 3, 5, 4, 3}, 3, 2000, 30, true, true); }

// ADF on rank-one measurements: <x, u_1 (x) ... (x) u_d> with Gaussian vectors u_k
// (RankOneMeasurementSet::random draws them with Tensor::random and sorts the samples).
static void case_adf_rankone() {
	reseed();
	const std::vector<size_t> dims{4, 5, 4, 5};
	TTTensor target = TTTensor::random(dims, 2);
	RankOneMeasurementSet m = RankOneMeasurementSet::random(300, target);
	TTTensor x = TTTensor::random(dims, 2);
	save_tt("target", target);
	save_tt("x0", x);
	std::vector<double> vec;
	for (auto& p : m.positions)
		for (auto& t : p) {
			Tensor u = t;
			u.use_dense_representation();
			for (size_t i = 0; i < u.size; ++i) vec.push_back(u[i]);
		}
	size_t sum_n = 0;
	for (auto n : dims) sum_n += n;
	save("vectors", vec, {m.size(), sum_n});
	save("values", m.measuredValues);
	PerformanceData perf(false, true);
	ADFVariant adf(25, 0.0, 1.0);
	const double res = adf(x, m, perf);
	save("perf_residual", perf_residuals(perf));
	save_scalar("final_residual", res);
	save_tt("x_final", x);
	auto pos = probe_positions(dims, 100, 31);
	save_probes("x_final", x, pos);
}
static void case_adf_cfg5() { adf_case("cfg5", std::vector<size_t>(10, 8), 6, 200000, 50, false, true); }

// ADF with rank increase: the ADFVariant::operator() overload taking maxRanks
// (adf.h:263-266, adf.cpp:590-602). x starts at rank 1 below a rank-3 target;
// each stagnation (minimal decrease 0.99) adds a 1e-6-scaled rank-1 random TT
// (target residual 1e-10, above the rounding floor)
// drawn from the library's random state and rounds to maxRanks. The random state
// is reseeded with 0x5EED right before the call so the device can replay it.
static void case_adf_rankinc() {
	reseed();
	const std::vector<size_t> dims{4, 5, 3, 5, 4, 3};
	TTTensor target = TTTensor::random(dims, 3);
	const size_t N = 1500;
	SinglePointMeasurementSet m = SinglePointMeasurementSet::random(N, dims);
	m.measure(target);
	TTTensor x = TTTensor::random(dims, 1);
	save_tt("x0", x);
	std::vector<int64_t> pos;
	for (auto& p : m.positions)
		for (auto i : p) pos.push_back(int64_t(i));
	save("positions", pos, {N, dims.size()});
	save("values", m.measuredValues);
	const std::vector<size_t> maxRanks(dims.size() - 1, 3);
	misc::randomEngine.seed(0x5EED);
	misc::defaultNormalDistribution.reset();
	PerformanceData perf(false, true);
	ADFVariant adf(120, 1e-10, 0.99);
	const double res = adf(x, m, maxRanks, perf);
	std::vector<int64_t> iters, ranks;
	for (auto& dp : perf.data) {
		iters.push_back(int64_t(dp.iterationCount));
		for (auto r : dp.ranks) ranks.push_back(int64_t(r));
	}
	save("perf_residual", perf_residuals(perf));
	save("perf_iteration", iters);
	save("perf_ranks", ranks, {perf.data.size(), dims.size() - 1});
	save_scalar("final_residual", res);
	save_tt("x_final", x);
	save_probes("x_final", x, probe_positions(dims, 100, 37));
}

// Rank-revealing QC / CQ with a clear gap: z = x (+) s w stacks x and a scaled
// independent TT w in block cores (the sum x + s w). With s = 1e-10 the w part's
// R_kk sit at 1e-13..1e-11 R_00, far above the cutoff 16 eps R_00 and far above
// rounding, so they are kept; with s = 1e-17 they sit far below the cutoff and are
// dropped wherever R_00 > 0 (blasLapackWrapper.cpp:269,343 compare with the signed
// R_00). Either way the rank decision does not depend on rounding.
static TTTensor block_sum2(const TTTensor& x, const TTTensor& w, double s) {
	const size_t d = x.degree();
	TTTensor z(x.dimensions);
	for (size_t k = 0; k < d; ++k) {
		Tensor a = x.get_component(k), b = w.get_component(k);
		a.use_dense_representation();
		b.use_dense_representation();
		const size_t ra0 = a.dimensions[0], n = a.dimensions[1], ra1 = a.dimensions[2];
		const size_t rb0 = b.dimensions[0], rb1 = b.dimensions[2];
		const size_t R0 = k == 0 ? 1 : ra0 + rb0, R1 = k + 1 == d ? 1 : ra1 + rb1;
		Tensor c({R0, n, R1}, Tensor::Representation::Dense);
		for (size_t i = 0; i < ra0; ++i)
			for (size_t j = 0; j < n; ++j)
				for (size_t l = 0; l < ra1; ++l) c[(i * n + j) * R1 + l] = a[(i * n + j) * ra1 + l];
		const size_t o0 = k == 0 ? 0 : ra0, o1 = k + 1 == d ? 0 : ra1;
		for (size_t i = 0; i < rb0; ++i)
			for (size_t j = 0; j < n; ++j)
				for (size_t l = 0; l < rb1; ++l)
					c[((o0 + i) * n + j) * R1 + o1 + l] += (k == 0 ? s : 1.0) * b[(i * n + j) * rb1 + l];
		z.set_component(k, c);
	}
	return z;
}

// Rescales every bond of z by a diagonal D (core k times D on its right index, core k+1
// times D^-1 on its left): the same tensor, but no core has orthonormal rows or columns,
// so the pivoted factorisations never choose between columns of equal norm (random TTs
// come right-orthogonalised, whose equal column norms make the pivot order a matter of
// rounding).
static void rescale_bonds(TTTensor& z, uint64_t seed) {
	std::mt19937_64 rng(seed);
	std::uniform_real_distribution<double> u(0.5, 2.0);
	const size_t d = z.degree();
	for (size_t k = 0; k + 1 < d; ++k) {
		Tensor a = z.get_component(k), b = z.get_component(k + 1);
		a.use_dense_representation();
		b.use_dense_representation();
		const size_t r = a.dimensions[2], na = a.dimensions[0] * a.dimensions[1], nb = b.dimensions[1] * b.dimensions[2];
		for (size_t j = 0; j < r; ++j) {
			const double f = u(rng);
			for (size_t i = 0; i < na; ++i) a[i * r + j] *= f;
			for (size_t i = 0; i < nb; ++i) b[j * nb + i] /= f;
		}
		z.set_component(k, a);
		z.set_component(k + 1, b);
	}
}

static void case_qc_gap() {
	reseed();
	const std::vector<size_t> dims{4, 3, 5, 4, 3, 4, 3};
	TTTensor x = TTTensor::random(dims, {3, 5, 6, 5, 4, 3});
	TTTensor w = TTTensor::random(dims, {2, 3, 3, 4, 2, 2});
	auto pos = probe_positions(dims, 100, 41);
	for (const auto& tag : {std::string("keep"), std::string("drop")}) {
		const double s = tag == "keep" ? 1e-10 : 1e-17;
		TTTensor z = block_sum2(x, w, s);
		rescale_bonds(z, 43);
		save_tt(tag + "_z", z);
		for (size_t p : {dims.size() - 1, size_t(0), size_t(3)}) {
			TTTensor y = z;
			y.move_core(p, false);
			save(tag + "_qc_to" + std::to_string(p) + "_ranks", ranks_of(y));
			save_probes(tag + "_qc_to" + std::to_string(p), y, pos);
		}
	}
}

// xerus's own binary file format (misc::save_to_file): the bytes of files written
// by the reference, with the numbers they hold, for byte-exact writer/reader tests.
static void save_file_bytes(const std::string& name, const std::string& path) {
	std::ifstream f(path, std::ios::binary);
	std::vector<uint8_t> bytes((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
	save(name, bytes);
}

static void case_fileio() {
	reseed();
	TTTensor x = TTTensor::random({3, 4, 2, 5}, {2, 7, 3});
	save_tt("x", x);
	misc::save_to_file(x, g_out + "/x.xrs");
	save_file_bytes("x_bytes", g_out + "/x.xrs");
	TTTensor y = x;
	y.move_core(2);
	save_tt("y", y);
	misc::save_to_file(y, g_out + "/y.xrs");
	save_file_bytes("y_bytes", g_out + "/y.xrs");
	TTTensor z = x + x;  // a sum is not canonical
	save_tt("z", z);
	save<int64_t>("z_canon", {int64_t(z.canonicalized), int64_t(z.corePosition)});
	misc::save_to_file(z, g_out + "/z.xrs");
	save_file_bytes("z_bytes", g_out + "/z.xrs");
	TTOperator A = laplace_operator(4, 3, nullptr, false);
	save_op("A", A);
	misc::save_to_file(A, g_out + "/A.xrs");
	save_file_bytes("A_bytes", g_out + "/A.xrs");
}

// IHT (algorithms/iht.cpp:29-155) on a small completion problem. The reference loops
// 10^6 iterations with no stopping test, so the run is ended from the PerformanceData's
// error callback, which sees every iterate: it records the iterate's probes and, after
// the twelfth, throws. The recorded residuals are PerformanceData's (one per iteration).
struct StopIht {};
static void case_iht() {
	reseed();
	const std::vector<size_t> dims{4, 3, 4, 3, 4};
	TTTensor target = TTTensor::random(dims, 2);
	target /= frob_norm(target);
	const size_t N = 60;
	SinglePointMeasurementSet m = SinglePointMeasurementSet::random(N, dims);
	m.measure(target);
	TTTensor x = TTTensor::random(dims, 2);
	x /= frob_norm(x);
	save_tt("x0", x);
	std::vector<int64_t> pos;
	for (auto& p : m.positions)
		for (auto i : p) pos.push_back(int64_t(i));
	save("positions", pos, {N, dims.size()});
	save("values", m.measuredValues);
	const auto probes = probe_positions(dims, 80, 53);
	std::vector<double> probe_vals;
	std::vector<int64_t> probe_pos;
	for (auto& p : probes)
		for (auto i : p) probe_pos.push_back(int64_t(i));
	save("probe_pos", probe_pos, {probes.size(), dims.size()});
	size_t seen = 0;
	const size_t iters = 12;
	PerformanceData perf(
	    [&](const TTTensor& xi) -> double {
		    for (auto& p : probes) probe_vals.push_back(tt_entry(xi, p));
		    if (++seen >= iters) throw StopIht();
		    return 0.0;
	    },
	    false, true);
	try {
		IHT(x, m, perf);
	} catch (const StopIht&) {
	}
	save("perf_residual", perf_residuals(perf));
	save("probe_val", probe_vals, {seen, probes.size()});
}

// ------------------------------------------------------------------- timing
// The reference's own implementation timed on this host (wall clock around the
// algorithm call only; inputs drawn as in the golden cases, PerformanceData
// inactive). Each case writes <tag>_seconds (and workload facts) like the others.
using Clock = std::chrono::steady_clock;
static double secs(Clock::time_point a, Clock::time_point b) { return std::chrono::duration<double>(b - a).count(); }

// ALS_SPD on the d=8, n=4 Laplacian: rank 8 for 20 half-sweeps with convergenceEpsilon 0
// (the configuration as stated), and rank 32 for the two half-sweeps that reach 1e-8.
static void case_time_cfg1() {
	const size_t d = 8, n = 4;
	TTOperator A = laplace_operator(d, n, nullptr, false);
	for (size_t rank : {size_t(8), size_t(32)}) {
		reseed();
		TTTensor b = TTTensor::random(std::vector<size_t>(d, n), 4);
		TTTensor x = TTTensor::random(std::vector<size_t>(d, n), rank);
		x /= frob_norm(x);
		ALSVariant als = ALS_SPD;
		als.convergenceEpsilon = 0.0;
		const size_t hs = rank == 8 ? 20 : 2;
		auto t0 = Clock::now();
		als(A, x, b, hs);
		auto t1 = Clock::now();
		const std::string tag = "r" + std::to_string(rank) + "_hs" + std::to_string(hs);
		save_scalar(tag + "_seconds", secs(t0, t1));
		save_scalar(tag + "_residual", residual_of(A, x, b));
	}
}

// Configuration 2: move_core(d-1) (QC sweep), round(32) and the dot product on two
// independent d=32, n=4, rank-64 tensors with N(0, 1/8) entries.
static void case_time_cfg2() {
	reseed();
	std::normal_distribution<double> dist(0.0, 0.125);
	const std::vector<size_t> dims(32, 4);
	TTTensor x = TTTensor::random(dims, std::vector<size_t>(31, 64), dist, misc::randomEngine);
	TTTensor y = TTTensor::random(dims, std::vector<size_t>(31, 64), dist, misc::randomEngine);
	Index i;
	const int reps = 5;
	double tm = 0, tr = 0, td = 0;
	for (int rep = 0; rep < reps; ++rep) {
		TTTensor z = x;
		auto t0 = Clock::now();
		z.move_core(31);
		auto t1 = Clock::now();
		TTTensor w = x;
		auto t2 = Clock::now();
		w.round(size_t(32));
		auto t3 = Clock::now();
		const double v = value_t(x(i & 0) * y(i & 0));
		auto t4 = Clock::now();
		(void)v;
		tm += secs(t0, t1);
		tr += secs(t2, t3);
		td += secs(t3, t4);
	}
	save_scalar("move_core_seconds", tm / reps);
	save_scalar("round_seconds", tr / reps);
	save_scalar("dot_seconds", td / reps);
}

// Configuration 4: ALS_SPD, 4 sweeps, on a sample of the batch's instances (their
// shapes read from <outdir>/cfg4_params.txt: d n shift rhs_rank start_rank seed per
// line), one instance per OpenMP thread; instances per second over the sample.
static void case_time_cfg4() {
	std::ifstream f(g_out + "/cfg4_params.txt");
	struct P { size_t d, n; double shift; size_t rb, rx; uint64_t seed; };
	std::vector<P> ps;
	P p;
	while (f >> p.d >> p.n >> p.shift >> p.rb >> p.rx >> p.seed) ps.push_back(p);
	std::vector<TTOperator> As(ps.size());
	std::vector<TTTensor> xs(ps.size()), bs(ps.size());
	for (size_t q = 0; q < ps.size(); ++q) {
		misc::randomEngine.seed(ps[q].seed);
		misc::defaultNormalDistribution.reset();
		As[q] = laplace_operator(ps[q].d, ps[q].n, nullptr, false, ps[q].shift);
		bs[q] = TTTensor::random(std::vector<size_t>(ps[q].d, ps[q].n), ps[q].rb);
		xs[q] = TTTensor::random(std::vector<size_t>(ps[q].d, ps[q].n), ps[q].rx);
		xs[q] /= frob_norm(xs[q]);
	}
	ALSVariant als = ALS_SPD;
	als.convergenceEpsilon = 0.0;
	auto t0 = Clock::now();
#pragma omp parallel for schedule(dynamic, 1)
	for (size_t q = 0; q < ps.size(); ++q) als(As[q], xs[q], bs[q], size_t(8));
	auto t1 = Clock::now();
	save_scalar("sample_seconds", secs(t0, t1));
	save_scalar("sample_instances", double(ps.size()));
}

// Configuration 5: 50 ADF iterations, d=10, n=8, rank 6, 200 000 samples.
static void case_time_cfg5() {
	reseed();
	const std::vector<size_t> dims(10, 8);
	TTTensor target = TTTensor::random(dims, 6);
	SinglePointMeasurementSet m = SinglePointMeasurementSet::random(200000, dims);
	m.measure(target);
	std::normal_distribution<double> noise(0.0, 1e-6);
	for (auto& v : m.measuredValues) v += noise(misc::randomEngine);
	TTTensor x = TTTensor::random(dims, 6);
	ADFVariant adf(50, 0.0, 1.0);
	auto t0 = Clock::now();
	PerformanceData none(false, false);
	const double res = adf(x, m, none);
	auto t1 = Clock::now();
	save_scalar("adf50_seconds", secs(t0, t1));
	save_scalar("adf50_residual", res);
}

int main(int argc, char** argv) {
	if (argc != 3) {
		std::fprintf(stderr, "usage: %s <case> <outdir>\n", argv[0]);
		return 2;
	}
	g_out = argv[2];
	const std::string c = argv[1];
	if (c == "rng") case_rng();
	else if (c == "tt_random") case_tt_random();
	else if (c == "dot") case_dot();
	else if (c == "movecore") case_movecore();
	else if (c == "round") case_round();
	else if (c == "als") case_als();
	else if (c == "dmrg") case_dmrg();
	else if (c == "adf") case_adf();
	else if (c == "adf_cfg5") case_adf_cfg5();
	else if (c == "fileio") case_fileio();
	else if (c == "als_nonspd") case_als_nonspd();
	else if (c == "arith") case_arith();
	else if (c == "adf_rankone") case_adf_rankone();
	else if (c == "gcg") case_gcg();
	else if (c == "adf_rankinc") case_adf_rankinc();
	else if (c == "qc_gap") case_qc_gap();
	else if (c == "retractions") case_retractions();
	else if (c == "iht") case_iht();
	else if (c == "time_cfg1") case_time_cfg1();
	else if (c == "time_cfg2") case_time_cfg2();
	else if (c == "time_cfg4") case_time_cfg4();
	else if (c == "time_cfg5") case_time_cfg5();
	else {
		std::fprintf(stderr, "unknown case %s\n", c.c_str());
		return 2;
	}
	return 0;
}
