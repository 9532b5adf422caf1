// extern "C" entry points of libxtt.so (declared in include/xtt.h): argument
// checks, exception-to-status translation, the host random state, and the
// calls into the engine.
#include <algorithm>
#include <cstring>
#include <new>
#include <random>
#include <set>
#include <string>

#include <vector>

#include "als.cuh"

namespace {

thread_local std::string g_error;
thread_local std::mt19937_64 g_engine;                   // analogue of xerus::misc::randomEngine
thread_local std::normal_distribution<double> g_normal;  // analogue of xerus::misc::defaultNormalDistribution
thread_local std::normal_distribution<double> g_custom;  // last non-default N(mean, stddev), reused while unchanged

template <class F>
int guard(F&& f) {
	try {
		f();
		g_error.clear();
		return XTT_OK;
	} catch (const xtt::Error& e) {
		g_error = e.what();
		return e.code;
	} catch (const std::bad_alloc&) {
		g_error = "host allocation failed";
		return XTT_ERR_NO_MEMORY;
	} catch (const std::exception& e) {
		g_error = e.what();
		return XTT_ERR_ARGUMENT;
	}
}

std::normal_distribution<double>& dist_for(double mean, double stddev) {
	if (mean == 0.0 && stddev == 1.0) return g_normal;
	if (g_custom.mean() != mean || g_custom.stddev() != stddev) g_custom = std::normal_distribution<double>(mean, stddev);
	return g_custom;
}

// TTNetwork::random's fill (include/xerus/ttNetwork.h:128-155): every core in order,
// row-major, one draw per entry from the library engine, then move_core(0) with
// rank-revealing QR. t has its (maximal-reduced) ranks already.
void fill_random(xtt::Tensor& t, double mean, double stddev) {
	auto& dist = dist_for(mean, stddev);
	std::vector<double> host;
	for (int k = 0; k < t.d; ++k) {
		host.resize(t.core_size(k));
		for (auto& v : host) v = dist(g_engine);
		XTT_CUDA(cudaMemcpyAsync(t.core[k], host.data(), host.size() * sizeof(double), cudaMemcpyHostToDevice,
		                         t.ctx->stream));
		XTT_CUDA(cudaStreamSynchronize(t.ctx->stream));
	}
	t.canonicalized = (t.d == 1);
	t.core_position = 0;
	xtt::move_core(t, 0, false);
	t.ctx->sync();
}

}  // namespace

namespace xtt {
// Lets entry points outside this file leave a message for xtt_last_error().
void set_last_error(const std::string& msg) { g_error = msg; }
}  // namespace xtt

struct xtt_context {
	xtt::Context* c;
};
struct xtt_tensor {
	xtt::Tensor* t;
};

#define ARG(cond, msg) XTT_REQUIRE(cond, msg)

extern "C" {

const char* xtt_last_error(void) { return g_error.c_str(); }
const char* xtt_version(void) { return "xtt 0.1 (GB300 sm_103a; xerus 3.0.1 sweep path)"; }

int xtt_context_create(int device, xtt_context** out) {
	return guard([&] {
		ARG(out, "out is NULL");
		*out = nullptr;
		xtt::DeviceScope dev_scope(device);
		auto* c = new xtt::Context(device);
		*out = new xtt_context{c};
	});
}

// A context is freed only after its last tensor: tensor destructors use its
// stream, and callers (garbage-collected bindings in particular) may destroy
// them in any order.
static void release_context(xtt::Context* c) {
	if (c->closing && c->tensors == 0) delete c;
}

int xtt_context_destroy(xtt_context* ctx) {
	return guard([&] {
		xtt::DeviceScope dev_scope(ctx ? ctx->c->device : -1);
		if (!ctx) return;
		ctx->c->closing = true;
		release_context(ctx->c);
		delete ctx;
	});
}

int xtt_context_set_stream(xtt_context* ctx, void* stream) {
	return guard([&] {
		xtt::DeviceScope dev_scope(ctx ? ctx->c->device : -1);
		ARG(ctx, "ctx is NULL");
		XTT_CUDA(cudaStreamSynchronize(ctx->c->stream));
		ctx->c->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->c->own;
	});
}

int xtt_context_synchronize(xtt_context* ctx) {
	return guard([&] {
		xtt::DeviceScope dev_scope(ctx ? ctx->c->device : -1);
		ARG(ctx, "ctx is NULL");
		ctx->c->sync();
	});
}

int xtt_context_kernel_launches(xtt_context* ctx, int64_t* count) {
	return guard([&] {
		xtt::DeviceScope dev_scope(ctx ? ctx->c->device : -1);
		ARG(ctx && count, "NULL argument");
		*count = ctx->c->launches;
	});
}

int xtt_context_profile(xtt_context* ctx, int enable) {
	return guard([&] {
		xtt::DeviceScope dev_scope(ctx ? ctx->c->device : -1);
		ARG(ctx, "ctx is NULL");
		xtt::Context& c = *ctx->c;
		c.resolve_profile();
		if (enable) c.profile.clear();
		c.profiling = enable != 0;
	});
}

int xtt_context_profile_work(xtt_context* ctx, const char* name, double* bytes, double* flops) {
	return guard([&] {
		xtt::DeviceScope dev_scope(ctx ? ctx->c->device : -1);
		ARG(ctx && name && bytes && flops, "NULL argument");
		xtt::Context& c = *ctx->c;
		c.resolve_profile();
		*bytes = 0;
		*flops = 0;
		for (auto& e : c.profile)
			if (e.first == name) {
				*bytes = e.second.bytes;
				*flops = e.second.flops;
			}
	});
}

int xtt_context_set_cg_path(xtt_context* ctx, int path) {
	return guard([&] {
		xtt::DeviceScope dev_scope(ctx ? ctx->c->device : -1);
		ARG(ctx, "ctx is NULL");
		ARG(path == XTT_CG_PATH_AUTO || path == XTT_CG_PATH_GRID || path == XTT_CG_PATH_TENSOR, "unknown CG path");
		ctx->c->cg_path = path;
	});
}

int xtt_gemm_tc(xtt_context* ctx, int64_t m, int64_t n, int64_t k, const double* A, int64_t lda, const double* B,
                int64_t ldb, double* C, int64_t ldc, int32_t terms) {
	return guard([&] {
		xtt::DeviceScope dev_scope(ctx ? ctx->c->device : -1);
		ARG(ctx && A && B && C, "NULL argument");
		ARG(m > 0 && n > 0 && k > 0 && m < (1 << 30) && n < (1 << 30) && k < (1 << 30), "illegal GEMM size");
		ARG(lda >= k && ldb >= n && ldc >= n, "leading dimension smaller than the row");
		ARG(terms == 1 || terms == 2 || terms == 3 || terms == 6, "terms must be 1, 2, 3 or 6");
		xtt::Gemm<double> g;
		g.M = int(m); g.N = int(n); g.K = int(k);
		g.A = A; g.sAm = lda; g.sAk = 1;
		g.B = B; g.sBk = ldb; g.sBn = 1;
		g.C = C; g.sCm = ldc; g.sCn = 1;
		g.lens((m - 1) * lda + k, (k - 1) * ldb + n, (m - 1) * ldc + n);
		if (terms == 2) xtt::gemm_df(*ctx->c, g);
		else xtt::gemm_tc(*ctx->c, g, terms);
	});
}

int xtt_context_set_contraction_precision(xtt_context* ctx, int terms) {
	return guard([&] {
		xtt::DeviceScope dev_scope(ctx ? ctx->c->device : -1);
		ARG(ctx, "ctx is NULL");
		ARG(terms == 0 || terms == 1 || terms == 3 || terms == 6,
		    "contraction precision must be 0 (FP64), 3 (split TF32), 6 (split BF16) or 1 (TF32)");
		ctx->c->contraction_terms = terms;
	});
}

int xtt_context_set_svd_path(xtt_context* ctx, int path) {
	return guard([&] {
		xtt::DeviceScope dev_scope(ctx ? ctx->c->device : -1);
		ARG(ctx, "ctx is NULL");
		ARG(path == XTT_SVD_PATH_AUTO || path == XTT_SVD_PATH_JACOBI, "unknown SVD path");
		ctx->c->svd_path = path;
	});
}

int xtt_context_profile_get(xtt_context* ctx, const char* name, int64_t* launches, double* milliseconds) {
	return guard([&] {
		xtt::DeviceScope dev_scope(ctx ? ctx->c->device : -1);
		ARG(ctx && name && launches && milliseconds, "NULL argument");
		xtt::Context& c = *ctx->c;
		c.resolve_profile();
		*launches = 0;
		*milliseconds = 0;
		for (auto& e : c.profile)
			if (e.first == name) {
				*launches = e.second.launches;
				*milliseconds = e.second.ms;
			}
	});
}

int xtt_tensor_create(xtt_context* ctx, int is_operator, int64_t order, const int64_t* dims, const int64_t* ranks,
                      xtt_tensor** out) {
	return guard([&] {
		xtt::DeviceScope dev_scope(ctx ? ctx->c->device : -1);
		ARG(ctx && dims && ranks && out, "NULL argument");
		ARG(order > 0 && order < (1 << 20), "order must be positive");
		*out = nullptr;
		auto* t = new xtt::Tensor(ctx->c, is_operator != 0, int(order), dims, ranks);
		ctx->c->tensors++;
		*out = new xtt_tensor{t};
	});
}

int xtt_tensor_destroy(xtt_tensor* t) {
	return guard([&] {
		xtt::DeviceScope dev_scope(t ? t->t->ctx->device : -1);
		if (!t) return;
		xtt::Context* c = t->t->ctx;
		delete t->t;
		delete t;
		c->tensors--;
		release_context(c);
	});
}

int xtt_tensor_copy(const xtt_tensor* src, xtt_tensor** out) {
	return guard([&] {
		xtt::DeviceScope dev_scope(src ? src->t->ctx->device : -1);
		ARG(src && out, "NULL argument");
		const xtt::Tensor& s = *src->t;
		auto* t = new xtt::Tensor(s.ctx, s.op, s.d, s.dims.data(), s.ranks.data());
		s.ctx->tensors++;
		*out = new xtt_tensor{t};
		t->copy_from(s);
	});
}

int xtt_tensor_order(const xtt_tensor* t, int64_t* order) {
	return guard([&] {
		ARG(t && order, "NULL argument");
		*order = t->t->d;
	});
}

int xtt_tensor_dims(const xtt_tensor* t, int64_t* dims) {
	return guard([&] {
		ARG(t && dims, "NULL argument");
		std::copy(t->t->dims.begin(), t->t->dims.end(), dims);
	});
}

int xtt_tensor_ranks(const xtt_tensor* t, int64_t* ranks) {
	return guard([&] {
		ARG(t && ranks, "NULL argument");
		std::copy(t->t->ranks.begin(), t->t->ranks.end(), ranks);
	});
}

int xtt_tensor_size(const xtt_tensor* t, int64_t* count) {
	return guard([&] {
		ARG(t && count, "NULL argument");
		*count = int64_t(t->t->total_size());
	});
}

int xtt_tensor_set_cores(xtt_tensor* t, const double* host, int64_t count) {
	return guard([&] {
		xtt::DeviceScope dev_scope(t ? t->t->ctx->device : -1);
		ARG(t && host, "NULL argument");
		xtt::Tensor& x = *t->t;
		ARG(count == int64_t(x.total_size()), "count does not match the tensor size");
		size_t off = 0;
		for (int k = 0; k < x.d; ++k) {
			XTT_CUDA(cudaMemcpyAsync(x.core[k], host + off, x.core_size(k) * sizeof(double), cudaMemcpyHostToDevice,
			                         x.ctx->stream));
			off += x.core_size(k);
		}
		x.ctx->sync();
		x.canonicalized = false;
	});
}

int xtt_tensor_get_cores(const xtt_tensor* t, double* host, int64_t count) {
	return guard([&] {
		xtt::DeviceScope dev_scope(t ? t->t->ctx->device : -1);
		ARG(t && host, "NULL argument");
		const xtt::Tensor& x = *t->t;
		ARG(count == int64_t(x.total_size()), "count does not match the tensor size");
		size_t off = 0;
		for (int k = 0; k < x.d; ++k) {
			XTT_CUDA(cudaMemcpyAsync(host + off, x.core[k], x.core_size(k) * sizeof(double), cudaMemcpyDeviceToHost,
			                         x.ctx->stream));
			off += x.core_size(k);
		}
		x.ctx->sync();
	});
}

int xtt_file_encode(int is_operator, int64_t order, const int64_t* dims, const int64_t* ranks, const double* cores,
                    int canonicalized, int64_t core_position, uint8_t* buffer, int64_t capacity, int64_t* size) {
	return guard([&] {
		ARG(dims && ranks && cores && size, "NULL argument");
		ARG(order > 0 && order < (1 << 20), "order must be positive");
		std::vector<int64_t> dv(dims, dims + order), rv(ranks, ranks + order + 1);
		const std::vector<uint8_t> b = xtt::tt_file_encode(is_operator != 0, dv, rv, cores, canonicalized != 0,
		                                                   core_position);
		*size = int64_t(b.size());
		if (buffer) {
			ARG(capacity >= int64_t(b.size()), "buffer too small");
			std::memcpy(buffer, b.data(), b.size());
		}
	});
}

int xtt_file_decode(const uint8_t* buffer, int64_t size, int* is_operator, int64_t* order, int64_t* dims,
                    int64_t* ranks, int64_t dims_capacity, double* cores, int64_t cores_capacity, int64_t* cores_count,
                    int* canonicalized, int64_t* core_position) {
	return guard([&] {
		ARG(buffer && size >= 0 && is_operator && order && cores_count && canonicalized && core_position,
		    "NULL argument");
		const xtt::TtFile f = xtt::tt_file_decode(buffer, size_t(size));
		*is_operator = f.op ? 1 : 0;
		*order = int64_t(f.dims.size());
		*cores_count = int64_t(f.cores.size());
		*canonicalized = f.canonicalized ? 1 : 0;
		*core_position = f.core_position;
		if (dims && ranks) {
			ARG(dims_capacity >= int64_t(f.dims.size()), "dims capacity too small");
			std::copy(f.dims.begin(), f.dims.end(), dims);
			std::copy(f.ranks.begin(), f.ranks.end(), ranks);
		}
		if (cores) {
			ARG(cores_capacity >= int64_t(f.cores.size()), "cores capacity too small");
			std::copy(f.cores.begin(), f.cores.end(), cores);
		}
	});
}

int xtt_tensor_save(const xtt_tensor* t, const char* path) {
	return guard([&] {
		xtt::DeviceScope dev_scope(t ? t->t->ctx->device : -1);
		ARG(t && path, "NULL argument");
		const xtt::Tensor& x = *t->t;
		std::vector<double> h(x.total_size());
		size_t off = 0;
		for (int k = 0; k < x.d; ++k) {
			XTT_CUDA(cudaMemcpyAsync(h.data() + off, x.core[k], x.core_size(k) * sizeof(double), cudaMemcpyDeviceToHost,
			                         x.ctx->stream));
			off += x.core_size(k);
		}
		x.ctx->sync();
		xtt::write_file(path, xtt::tt_file_encode(x.op, x.dims, x.ranks, h.data(), x.canonicalized, x.core_position));
	});
}

int xtt_tensor_load(xtt_context* ctx, const char* path, xtt_tensor** out) {
	return guard([&] {
		xtt::DeviceScope dev_scope(ctx ? ctx->c->device : -1);
		ARG(ctx && path && out, "NULL argument");
		*out = nullptr;
		const std::vector<uint8_t> b = xtt::read_file(path);
		const xtt::TtFile f = xtt::tt_file_decode(b.data(), b.size());
		auto* x = new xtt::Tensor(ctx->c, f.op, int(f.dims.size()), f.dims.data(), f.ranks.data());
		ctx->c->tensors++;
		auto* h = new xtt_tensor{x};
		try {
			size_t off = 0;
			for (int k = 0; k < x->d; ++k) {
				XTT_CUDA(cudaMemcpyAsync(x->core[k], f.cores.data() + off, x->core_size(k) * sizeof(double),
				                         cudaMemcpyHostToDevice, x->ctx->stream));
				off += x->core_size(k);
			}
			x->ctx->sync();
		} catch (...) {
			xtt_tensor_destroy(h);
			throw;
		}
		x->canonicalized = f.canonicalized;
		x->core_position = f.core_position;
		*out = h;
	});
}

int xtt_tensor_assign(xtt_tensor* t, const int64_t* ranks, const double* host, int64_t count) {
	return guard([&] {
		xtt::DeviceScope dev_scope(t ? t->t->ctx->device : -1);
		ARG(t && ranks && host, "NULL argument");
		xtt::Tensor& x = *t->t;
		ARG(ranks[0] == 1 && ranks[x.d] == 1, "boundary ranks must be 1");
		size_t total = 0;
		for (int k = 0; k < x.d; ++k) {
			ARG(ranks[k + 1] > 0, "rank 0 is not valid");
			total += size_t(ranks[k]) * x.n(k) * ranks[k + 1];
		}
		ARG(count == int64_t(total), "count does not match the ranks");
		for (int k = 0; k < x.d; ++k) x.reshape_core(k, ranks[k], ranks[k + 1]);
		size_t off = 0;
		for (int k = 0; k < x.d; ++k) {
			XTT_CUDA(cudaMemcpyAsync(x.core[k], host + off, x.core_size(k) * sizeof(double), cudaMemcpyHostToDevice,
			                         x.ctx->stream));
			off += x.core_size(k);
		}
		x.ctx->sync();
		x.canonicalized = false;
	});
}

int xtt_tensor_get_canonical(const xtt_tensor* t, int* canonicalized, int64_t* core_position) {
	return guard([&] {
		ARG(t && canonicalized && core_position, "NULL argument");
		*canonicalized = t->t->canonicalized ? 1 : 0;
		*core_position = t->t->core_position;
	});
}

int xtt_tensor_set_canonical(xtt_tensor* t, int canonicalized, int64_t core_position) {
	return guard([&] {
		ARG(t, "NULL argument");
		ARG(core_position >= 0 && core_position < t->t->d, "illegal core position");
		t->t->canonicalized = canonicalized != 0;
		t->t->core_position = core_position;
	});
}

int xtt_tensor_scale(xtt_tensor* t, double f) {
	return guard([&] {
		xtt::DeviceScope dev_scope(t ? t->t->ctx->device : -1);
		ARG(t, "NULL argument");
		xtt::Tensor& x = *t->t;
		const int k = x.canonicalized ? int(x.core_position) : 0;
		xtt::scale(*x.ctx, x.core[k], f, x.core_size(k));
		x.ctx->sync();
	});
}

int xtt_random_seed(uint64_t seed) {
	return guard([&] {
		g_engine.seed(seed);
		g_normal.reset();
		g_custom.reset();
	});
}

int xtt_random_normal(double mean, double stddev, int64_t count, double* out) {
	return guard([&] {
		ARG(out || count == 0, "NULL argument");
		auto& dist = dist_for(mean, stddev);
		for (int64_t i = 0; i < count; ++i) out[i] = dist(g_engine);
	});
}

int xtt_tensor_random(xtt_context* ctx, int64_t order, const int64_t* dims, const int64_t* inner_ranks, double mean,
                      double stddev, xtt_tensor** out) {
	return guard([&] {
		xtt::DeviceScope dev_scope(ctx ? ctx->c->device : -1);
		ARG(ctx && dims && out && (order == 1 || inner_ranks), "NULL argument");
		ARG(order > 0, "order must be positive");
		*out = nullptr;
		std::vector<int64_t> dv(dims, dims + order), inner(order > 1 ? inner_ranks : dims, order > 1 ? inner_ranks + order - 1 : dims);
		for (auto v : dv) ARG(v > 0, "Trying to construct a TTTensor with dimension 0 is not possible.");
		for (auto v : inner) ARG(v > 0, "Trying to construct random TTTensor with rank 0 is illegal.");
		auto red = xtt::reduce_to_maximal_ranks(inner, dv);
		std::vector<int64_t> r(order + 1, 1);
		for (int64_t k = 1; k < order; ++k) r[k] = red[k - 1];
		auto* t = new xtt::Tensor(ctx->c, false, int(order), dv.data(), r.data());
		ctx->c->tensors++;
		xtt_tensor* h = new xtt_tensor{t};
		try {
			fill_random(*t, mean, stddev);
		} catch (...) {
			delete t;
			delete h;
			ctx->c->tensors--;
			throw;
		}
		*out = h;
	});
}

int xtt_random_positions(int64_t num, int64_t order, const int64_t* dims, int64_t* out) {
	return guard([&] {
		ARG(dims && (out || num == 0) && order > 0, "NULL argument");
		double total = 1;
		for (int64_t k = 0; k < order; ++k) {
			ARG(dims[k] > 0, "dimension 0 is not valid");
			total *= double(dims[k]);
		}
		ARG(total >= double(num), "It's impossible to perform as many measurements as requested.");
		// SinglePointMeasurementSet::create_random_positions (measurments.cpp:222-248)
		std::vector<std::uniform_int_distribution<size_t>> idx;
		for (int64_t k = 0; k < order; ++k) idx.emplace_back(0, size_t(dims[k] - 1));
		std::set<size_t> seen;
		std::vector<std::vector<size_t>> pos;
		pos.reserve(size_t(num));
		std::vector<size_t> m(order);
		while (int64_t(pos.size()) < num) {
			size_t lin = 0;
			for (int64_t k = 0; k < order; ++k) {
				m[k] = idx[k](g_engine);
				lin = lin * size_t(dims[k]) + m[k];
			}
			if (seen.insert(lin).second) pos.push_back(m);
		}
		std::sort(pos.begin(), pos.end());
		for (int64_t s = 0; s < num; ++s)
			for (int64_t k = 0; k < order; ++k) out[s * order + k] = int64_t(pos[s][k]);
	});
}

int xtt_move_core(xtt_tensor* x, int64_t position, int keep_rank) {
	return guard([&] {
		xtt::DeviceScope dev_scope(x ? x->t->ctx->device : -1);
		ARG(x, "NULL argument");
		xtt::ContractionPrecisionScope ps(*x->t->ctx);
		xtt::GramQrScope gram(*x->t->ctx);
		xtt::move_core(*x->t, position, keep_rank != 0);
		x->t->ctx->sync();
	});
}

int xtt_round(xtt_tensor* x, const int64_t* max_ranks, double eps, double* spectra, int64_t spectra_capacity,
              int64_t* spectra_count) {
	return guard([&] {
		xtt::DeviceScope dev_scope(x ? x->t->ctx->device : -1);
		ARG(x && (max_ranks || x->t->d == 1), "NULL argument");
		std::vector<int64_t> mr(max_ranks, max_ranks + (x->t->d - 1));
		std::vector<double> sp;
		xtt::ContractionPrecisionScope ps(*x->t->ctx);
		xtt::round_tt(*x->t, mr, eps, spectra ? &sp : nullptr);
		x->t->ctx->sync();
		if (spectra) {
			const int64_t n = std::min<int64_t>(spectra_capacity, int64_t(sp.size()));
			std::copy(sp.begin(), sp.begin() + n, spectra);
			if (spectra_count) *spectra_count = int64_t(sp.size());
		}
	});
}

int xtt_dot(const xtt_tensor* x, const xtt_tensor* y, double* out) {
	return guard([&] {
		xtt::DeviceScope dev_scope(x ? x->t->ctx->device : -1);
		ARG(x && y && out, "NULL argument");
		ARG(x->t->ctx == y->t->ctx, "tensors belong to different contexts");
		xtt::ContractionPrecisionScope ps(*x->t->ctx);
		*out = xtt::dot(*x->t, *y->t);
	});
}

int xtt_frob_norm(const xtt_tensor* x, double* out) {
	return guard([&] {
		xtt::DeviceScope dev_scope(x ? x->t->ctx->device : -1);
		ARG(x && out, "NULL argument");
		*out = xtt::frob_norm(*x->t);
	});
}

int xtt_residual(const xtt_tensor* A, const xtt_tensor* x, const xtt_tensor* b, double* out) {
	return guard([&] {
		xtt::DeviceScope dev_scope(x ? x->t->ctx->device : -1);
		ARG(A && x && b && out, "NULL argument");
		*out = xtt::residual(*A->t, *x->t, *b->t);
	});
}

int xtt_entries(const xtt_tensor* x, const int64_t* positions, int64_t count, double* out) {
	return guard([&] {
		xtt::DeviceScope dev_scope(x ? x->t->ctx->device : -1);
		ARG(x && (count == 0 || (positions && out)), "NULL argument");
		xtt::entries(*x->t, positions, count, out);
	});
}

int xtt_als_default_options(xtt_als_options* o) {
	return guard([&] {
		ARG(o, "NULL argument");
		std::memset(o, 0, sizeof(*o));
		o->sites = 1;
		o->local_solver = 0;
		o->preserve_core_position = 1;
		o->precision = XTT_PRECISION_FP64;
		o->num_half_sweeps = 0;
		o->convergence_epsilon = 1e-6;
		o->local_tolerance = 1e-13;
		o->local_max_iterations = 0;
		o->residual_target = 0;
		o->record_residuals = 0;
		o->max_rank = 0;
		o->svd_epsilon = 0;
		o->exact_environment = 0;
		o->assume_spd = 1;
		o->use_residual = 0;
	});
}

static xtt::AlsOptions to_options(const xtt_als_options* opt) {
	xtt::AlsOptions o;
	o.sites = opt->sites;
	o.local_solver = opt->local_solver;
	o.preserve_core_position = opt->preserve_core_position != 0;
	o.precision = opt->precision;
	o.num_half_sweeps = opt->num_half_sweeps;
	o.convergence_epsilon = opt->convergence_epsilon;
	o.local_tolerance = opt->local_tolerance;
	o.local_max_iterations = opt->local_max_iterations;
	o.residual_target = opt->residual_target;
	o.record_residuals = opt->record_residuals != 0;
	o.max_rank = opt->max_rank;
	o.svd_epsilon = opt->svd_epsilon;
	o.exact_environment = opt->exact_environment != 0;
	o.assume_spd = opt->assume_spd != 0;
	o.use_residual = opt->use_residual != 0;
	return o;
}

int xtt_als_batch(xtt_context* ctx, int64_t count, const xtt_tensor* const* A, xtt_tensor* const* x,
                  const xtt_tensor* const* b, const xtt_als_options* opt, int autotune, double* energies,
                  int64_t* local_iterations, xtt_batch_report* report) {
	return guard([&] {
		xtt::DeviceScope dev_scope(ctx ? ctx->c->device : -1);
		ARG(ctx && A && x && b && opt, "NULL argument");
		ARG(count > 0 && count <= (int64_t(1) << 24), "count must be in 1..2^24");
		ARG(opt->assume_spd, "the batched sweep runs the SPD variant only");
		ARG(!opt->use_residual, "the batched sweep uses the energy criterion");
		ARG(opt->local_tolerance > 0 && opt->local_tolerance < 1, "local_tolerance must be in (0, 1)");
		ARG(opt->precision == XTT_PRECISION_FP64 || opt->precision == XTT_PRECISION_MIXED, "unknown precision");
		ARG(opt->record_residuals == 0 && opt->residual_target == 0, "batch: no residual traces or targets");
		std::vector<const xtt::Tensor*> av(count), bv(count);
		std::vector<xtt::Tensor*> xv(count);
		for (int64_t i = 0; i < count; ++i) {
			ARG(A[i] && x[i] && b[i], "NULL tensor in the batch");
			av[i] = A[i]->t;
			xv[i] = x[i]->t;
			bv[i] = b[i]->t;
		}
		xtt::BatchResult r = xtt::als_batch(*ctx->c, av, xv, bv, to_options(opt), autotune != 0);
		for (int64_t i = 0; i < count; ++i) {
			if (energies) energies[i] = r.energy[i];
			if (local_iterations) local_iterations[i] = r.iterations[i];
		}
		if (report) {
			report->milliseconds = r.ms;
			report->threads = r.threads;
			report->ctas_per_sm = r.ctas_per_sm;
			report->tile = r.tile;
			report->ctas = r.ctas;
		}
	});
}

int xtt_als(const xtt_tensor* A, xtt_tensor* x, const xtt_tensor* b, const xtt_als_options* opt,
            xtt_als_report* report, double* residual_trace, int64_t* flag_trace, double* energy_trace,
            int64_t trace_capacity) {
	return guard([&] {
		xtt::DeviceScope dev_scope(x ? x->t->ctx->device : -1);
		ARG(x && b && opt, "NULL argument");
		ARG(opt->local_tolerance > 0 && opt->local_tolerance < 1, "local_tolerance must be in (0, 1)");
		ARG(opt->precision == XTT_PRECISION_FP64 || opt->precision == XTT_PRECISION_MIXED, "unknown precision");
		xtt::AlsReport r = xtt::als(A ? A->t : nullptr, *x->t, *b->t, to_options(opt));
		if (report) {
			report->energy = r.energy;
			report->residual = r.residual;
			report->half_sweeps = r.half_sweeps;
			report->micro_steps = r.micro_steps;
			report->local_iterations = r.local_iterations;
			report->refinements = r.refinements;
			report->trace_count = int64_t(std::max(r.residuals.size(), r.energies.size()));
		}
		if (residual_trace)
			for (size_t i = 0; i < r.residuals.size() && int64_t(i) < trace_capacity; ++i) residual_trace[i] = r.residuals[i];
		if (flag_trace)
			for (size_t i = 0; i < r.flags.size() && int64_t(i) < trace_capacity; ++i) flag_trace[i] = r.flags[i];
		if (energy_trace)
			for (size_t i = 0; i < r.energies.size() && int64_t(i) < trace_capacity; ++i) energy_trace[i] = r.energies[i];
	});
}

int xtt_apply(const xtt_tensor* A, const xtt_tensor* x, xtt_tensor** out) {
	return guard([&] {
		xtt::DeviceScope dev_scope(x ? x->t->ctx->device : -1);
		ARG(A && x && out, "NULL argument");
		*out = nullptr;
		const xtt::Tensor& xs = *x->t;
		ARG(A->t->op, "A must be a TT operator");
		ARG(A->t->d == xs.d && A->t->dims == xs.dims, "operator and tensor dimensions differ");
		ARG(A->t->ctx == xs.ctx, "A and x live on different contexts");
		std::vector<int64_t> r(xs.d + 1);
		for (int k = 0; k <= xs.d; ++k) r[k] = A->t->ranks[k] * xs.ranks[k];
		auto* y = new xtt::Tensor(xs.ctx, xs.op, xs.d, xs.dims.data(), r.data());
		xs.ctx->tensors++;
		auto* h = new xtt_tensor{y};
		try {
			xtt::tt_apply(*A->t, xs, *y);
		} catch (...) {
			xtt_tensor_destroy(h);
			throw;
		}
		*out = h;
	});
}

int xtt_add(xtt_tensor* x, const xtt_tensor* y, double alpha) {
	return guard([&] {
		xtt::DeviceScope dev_scope(x ? x->t->ctx->device : -1);
		ARG(x && y, "NULL argument");
		ARG(x->t->ctx == y->t->ctx, "x and y live on different contexts");
		ARG(x != y, "x and y must be different tensors (copy y first)");
		xtt::tt_add(*x->t, *y->t, alpha);
	});
}

int xtt_als_energy_gradient(const xtt_tensor* A, const xtt_tensor* x, const xtt_tensor* b, double* energy,
                            double* grad, int64_t count) {
	return guard([&] {
		xtt::DeviceScope dev_scope(x ? x->t->ctx->device : -1);
		ARG(A && x && b && energy, "NULL argument");
		std::vector<double> g;
		*energy = xtt::als_energy_gradient(*A->t, *x->t, *b->t, g);
		if (grad) {
			ARG(count == int64_t(g.size()), "count does not match the tensor size");
			std::copy(g.begin(), g.end(), grad);
		}
	});
}

int xtt_adf(xtt_tensor* x, const int64_t* positions, const double* values, int64_t num, const xtt_adf_options* opt,
            double* final_residual, double* residual_trace, int64_t trace_capacity, int64_t* trace_count) {
	return guard([&] {
		xtt::DeviceScope dev_scope(x ? x->t->ctx->device : -1);
		ARG(x && positions && values && opt, "NULL argument");
		ARG(opt->precision == XTT_PRECISION_FP64 || opt->precision == XTT_PRECISION_MIXED, "unknown precision");
		xtt::AdfResult r = xtt::adf(*x->t, positions, values, num, opt->max_iterations, opt->target_residual,
		                            opt->min_decrease, opt->precision);
		x->t->ctx->sync();
		if (final_residual) *final_residual = r.checked_residual;
		if (residual_trace)
			for (size_t i = 0; i < r.trace.size() && int64_t(i) < trace_capacity; ++i) residual_trace[i] = r.trace[i];
		if (trace_count) *trace_count = int64_t(r.trace.size());
	});
}

int xtt_adf_max_ranks(xtt_tensor* x, const int64_t* positions, const double* values, int64_t num,
                      const int64_t* max_ranks, const xtt_adf_options* opt, double* final_residual,
                      double* residual_trace, int64_t* iteration_trace, int64_t* rank_trace, int64_t trace_capacity,
                      int64_t* trace_count) {
	return guard([&] {
		xtt::DeviceScope dev_scope(x ? x->t->ctx->device : -1);
		ARG(x && positions && values && opt && max_ranks, "NULL argument");
		ARG(opt->precision == XTT_PRECISION_FP64 || opt->precision == XTT_PRECISION_MIXED, "unknown precision");
		xtt::Tensor& t = *x->t;
		const std::vector<int64_t> mr(max_ranks, max_ranks + (t.d - 1));
		for (auto v : mr) ARG(v > 0, "maximal ranks must be positive");
		// adf.cpp:592-595: rnd = TTTensor::random(dims, 1) from the library's random state,
		// x += (1e-6 ||x||) rnd / ||rnd|| (the factor applied to rnd's core 0)
		auto add_random_rank_one = [](xtt::Tensor& xx) {
			const std::vector<int64_t> ones(size_t(xx.d) + 1, 1);
			xtt::Tensor rnd(xx.ctx, false, xx.d, xx.dims.data(), ones.data());
			fill_random(rnd, 0.0, 1.0);
			const double f = (1e-6 * xtt::frob_norm(xx)) * (1.0 / xtt::frob_norm(rnd));
			xtt::scale(*rnd.ctx, rnd.core[0], f, rnd.core_size(0));
			xtt::tt_add(xx, rnd, 1.0);
		};
		xtt::AdfResult r = xtt::adf(t, positions, values, num, opt->max_iterations, opt->target_residual,
		                            opt->min_decrease, opt->precision, &mr, add_random_rank_one);
		t.ctx->sync();
		if (final_residual) *final_residual = r.checked_residual;
		for (size_t i = 0; i < r.trace.size() && int64_t(i) < trace_capacity; ++i) {
			if (residual_trace) residual_trace[i] = r.trace[i];
			if (iteration_trace) iteration_trace[i] = r.trace_iteration[i];
			if (rank_trace) std::copy(r.trace_ranks[i].begin(), r.trace_ranks[i].end(), rank_trace + i * (t.d - 1));
		}
		if (trace_count) *trace_count = int64_t(r.trace.size());
	});
}

int xtt_iht(xtt_tensor* x, const int64_t* positions, const double* values, int64_t num, int64_t max_iterations,
            double* residual, double* residual_trace, int64_t trace_capacity, int64_t* trace_count) {
	return guard([&] {
		xtt::DeviceScope dev_scope(x ? x->t->ctx->device : -1);
		ARG(x && positions && values, "NULL argument");
		ARG(max_iterations >= 0, "max_iterations must be >= 0");
		xtt::Tensor& t = *x->t;
		for (int64_t s = 0; s < num; ++s)
			for (int k = 0; k < t.d; ++k)
				ARG(positions[s * t.d + k] >= 0 && positions[s * t.d + k] < t.dims[k], "measurement position out of range");
		const xtt::IhtResult r = xtt::iht(t, positions, values, num, max_iterations);
		if (residual) *residual = r.residual;
		if (residual_trace)
			for (size_t i = 0; i < r.trace.size() && int64_t(i) < trace_capacity; ++i) residual_trace[i] = r.trace[i];
		if (trace_count) *trace_count = int64_t(r.trace.size());
	});
}

static int riemann_call(bool cg, const xtt_tensor* A, xtt_tensor* x, const xtt_tensor* b, int64_t num_steps,
                        double convergence_epsilon, int assume_spd, int retraction, double* residual,
                        double* residual_trace, int64_t trace_capacity, int64_t* trace_count) {
	return guard([&] {
		xtt::DeviceScope dev_scope(x ? x->t->ctx->device : -1);
		ARG(x && b, "NULL argument");
		ARG(num_steps >= 0, "num_steps must be >= 0");
		ARG(retraction == XTT_RETRACTION_SUBMANIFOLD || retraction == XTT_RETRACTION_HOSVD ||
		        retraction == XTT_RETRACTION_ALS,
		    "unknown retraction");
		const xtt::RiemannReport r =
		    cg ? xtt::geometric_cg(A ? A->t : nullptr, *x->t, *b->t, num_steps, convergence_epsilon, assume_spd != 0,
		                           retraction)
		       : xtt::steepest_descent(A ? A->t : nullptr, *x->t, *b->t, num_steps, convergence_epsilon,
		                               assume_spd != 0, retraction);
		if (residual) *residual = r.residual;
		if (residual_trace)
			for (size_t i = 0; i < r.trace.size() && int64_t(i) < trace_capacity; ++i) residual_trace[i] = r.trace[i];
		if (trace_count) *trace_count = int64_t(r.trace.size());
	});
}

int xtt_geometric_cg(const xtt_tensor* A, xtt_tensor* x, const xtt_tensor* b, int64_t num_steps,
                     double convergence_epsilon, int assume_spd, double* residual, double* residual_trace,
                     int64_t trace_capacity, int64_t* trace_count) {
	return riemann_call(true, A, x, b, num_steps, convergence_epsilon, assume_spd, XTT_RETRACTION_SUBMANIFOLD, residual,
	                    residual_trace, trace_capacity, trace_count);
}

int xtt_steepest_descent(const xtt_tensor* A, xtt_tensor* x, const xtt_tensor* b, int64_t num_steps,
                         double convergence_epsilon, int assume_spd, double* residual, double* residual_trace,
                         int64_t trace_capacity, int64_t* trace_count) {
	return riemann_call(false, A, x, b, num_steps, convergence_epsilon, assume_spd, XTT_RETRACTION_SUBMANIFOLD, residual,
	                    residual_trace, trace_capacity, trace_count);
}

int xtt_geometric_cg_retraction(const xtt_tensor* A, xtt_tensor* x, const xtt_tensor* b, int64_t num_steps,
                                double convergence_epsilon, int assume_spd, int retraction, double* residual,
                                double* residual_trace, int64_t trace_capacity, int64_t* trace_count) {
	return riemann_call(true, A, x, b, num_steps, convergence_epsilon, assume_spd, retraction, residual, residual_trace,
	                    trace_capacity, trace_count);
}

int xtt_steepest_descent_retraction(const xtt_tensor* A, xtt_tensor* x, const xtt_tensor* b, int64_t num_steps,
                                    double convergence_epsilon, int assume_spd, int retraction, double* residual,
                                    double* residual_trace, int64_t trace_capacity, int64_t* trace_count) {
	return riemann_call(false, A, x, b, num_steps, convergence_epsilon, assume_spd, retraction, residual,
	                    residual_trace, trace_capacity, trace_count);
}

int xtt_random_rank_one(int64_t num, int64_t order, const int64_t* dims, double* out) {
	return guard([&] {
		ARG(dims && (out || num == 0) && order > 0, "NULL argument");
		double total = 1;
		int64_t sum_n = 0;
		for (int64_t k = 0; k < order; ++k) {
			ARG(dims[k] > 0, "dimension 0 is not valid");
			total *= double(dims[k]);
			sum_n += dims[k];
		}
		ARG(total >= double(num), "It's impossible to perform as many measurements as requested.");
		// RankOneMeasurementSet::create_random_positions (measurments.cpp:522-544): a
		// Tensor::random({n}) per sample and mode from the default normal distribution, then
		// sort(true) with internal::comp (measurments.cpp:330-347, 549-...): mode by mode,
		// entry by entry, the larger value first
		auto& dist = dist_for(0.0, 1.0);
		std::vector<std::vector<double>> rows(static_cast<size_t>(num), std::vector<double>(static_cast<size_t>(sum_n)));
		for (auto& r : rows)
			for (auto& v : r) v = dist(g_engine);
		std::stable_sort(rows.begin(), rows.end(), [](const std::vector<double>& a, const std::vector<double>& b) {
			for (size_t i = 0; i < a.size(); ++i) {
				if (a[i] > b[i]) return true;
				if (a[i] < b[i]) return false;
			}
			return false;
		});
		for (int64_t s = 0; s < num; ++s) std::copy(rows[s].begin(), rows[s].end(), out + s * sum_n);
	});
}

int xtt_entries_rank_one(const xtt_tensor* x, const double* vectors, int64_t count, double* out) {
	return guard([&] {
		xtt::DeviceScope dev_scope(x ? x->t->ctx->device : -1);
		ARG(x && (count == 0 || (vectors && out)), "NULL argument");
		xtt::entries_rank_one(*x->t, vectors, count, out);
	});
}

int xtt_adf_rank_one(xtt_tensor* x, const double* vectors, const double* values, int64_t num,
                     const xtt_adf_options* opt, double* final_residual, double* residual_trace,
                     int64_t trace_capacity, int64_t* trace_count) {
	return guard([&] {
		xtt::DeviceScope dev_scope(x ? x->t->ctx->device : -1);
		ARG(x && vectors && values && opt, "NULL argument");
		ARG(opt->precision == XTT_PRECISION_FP64, "rank-one ADF runs in FP64");
		xtt::AdfResult r = xtt::adf_rank_one(*x->t, vectors, values, num, opt->max_iterations, opt->target_residual,
		                                     opt->min_decrease);
		x->t->ctx->sync();
		if (final_residual) *final_residual = r.checked_residual;
		if (residual_trace)
			for (size_t i = 0; i < r.trace.size() && int64_t(i) < trace_capacity; ++i) residual_trace[i] = r.trace[i];
		if (trace_count) *trace_count = int64_t(r.trace.size());
	});
}

int xtt_adf_gradient(const xtt_tensor* x, const int64_t* positions, const double* values, int64_t num, double* loss,
                     double* grad, int64_t count) {
	return guard([&] {
		xtt::DeviceScope dev_scope(x ? x->t->ctx->device : -1);
		ARG(x && positions && values && loss, "NULL argument");
		std::vector<double> g;
		*loss = xtt::adf_gradient(*x->t, positions, values, num, g);
		if (grad) {
			ARG(count == int64_t(g.size()), "count does not match the tensor size");
			std::copy(g.begin(), g.end(), grad);
		}
	});
}

}  // extern "C"
