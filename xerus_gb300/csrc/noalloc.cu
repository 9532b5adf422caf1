// Allocation-free TT dot product: xtt_dot_noalloc.
//
// Who needs it: callers that must not allocate device memory themselves or
// through this library. Typical cases are frameworks whose caching allocator
// has already reserved the device memory it manages (a cudaMalloc from a
// library can fail or fragment that pool), and latency-critical paths where
// cudaMalloc/cudaFree are too slow or where cudaFree's implicit device-wide
// synchronisation would stall other streams. Such callers pass device pointers
// to the cores and to the result and get the same contraction as xtt_dot.
//
// How: the zipper's intermediates live in g_zip_scratch, a file-scope
// __device__ array that exists once per device for as long as the library is
// loaded. Host code cannot use the array's name as a device address, so the
// first call on a device looks the address up with cudaGetSymbolAddress (with
// that device current) and caches it; that first call should therefore happen
// before any stream capture on that device. Every call writes all scratch it
// reads (the running 1x1 start value is set by the first kernel), so no state
// carries over between calls; but all calls share the one array, so calls
// whose kernels overlap on the GPU (concurrent streams or host threads) race
// and must be serialised by the caller.
//
// Limits: order >= 1, every rank <= 128, every mode size <= 16 (the scratch is
// 2 x 128^2 + 128*16*128 doubles = 2.25 MiB). Larger inputs are rejected with
// XTT_ERR_CAPACITY before anything is launched.
#include <mutex>
#include <string>

#include "common.cuh"

namespace xtt {
void set_last_error(const std::string& msg);
}

namespace {

constexpr int kNoAllocMaxRank = 128;
constexpr int kNoAllocMaxDim = 16;
constexpr size_t kZipM = size_t(kNoAllocMaxRank) * kNoAllocMaxRank;
constexpr size_t kZipT = size_t(kNoAllocMaxRank) * kNoAllocMaxDim * kNoAllocMaxRank;
constexpr size_t kZipScratchDoubles = 2 * kZipM + kZipT;

static __device__ __align__(256) double g_zip_scratch[kZipScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_zip_scratch on `device`, looked up once per device and kept for
// the life of the process: a cudaDeviceReset (or a reset of the primary context) after
// the first call on a device is not supported, the cached address would be stale.
double* scratch_on(int device, cudaError_t& err) {
	std::lock_guard<std::mutex> lock(g_setup_mutex);
	err = cudaSuccess;
	if (g_scratch_ptr[device]) return g_scratch_ptr[device];
	int prev = -1;
	err = cudaGetDevice(&prev);
	if (err != cudaSuccess) return nullptr;
	if (prev != device && (err = cudaSetDevice(device)) != cudaSuccess) return nullptr;
	void* p = nullptr;
	err = cudaGetSymbolAddress(&p, g_zip_scratch);
	if (prev != device) cudaSetDevice(prev);
	if (err != cudaSuccess) return nullptr;
	g_scratch_ptr[device] = static_cast<double*>(p);
	return g_scratch_ptr[device];
}

__global__ void k_zip_start(double* M) { M[0] = 1.0; }

// T[b][(i, a')] = sum_a M[a][b] x[a][(i, a')]        (T: ry x n x rx1)
__global__ void k_zip_left(const double* M, const double* x, double* T, int rx, int ry, int n, int rx1) {
	const long long total = (long long)ry * n * rx1, row = (long long)n * rx1;
	for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
		const long long b = e / row, rem = e - b * row;
		double s = 0.0;
		for (int a = 0; a < rx; ++a) s += M[(long long)a * ry + b] * x[a * row + rem];
		T[e] = s;
	}
}

// M'[a'][b'] = sum_{(b, i)} T[(b, i)][a'] y[(b, i)][b']   (M': rx1 x ry1)
__global__ void k_zip_right(const double* T, const double* y, double* M, int ry, int n, int rx1, int ry1) {
	const long long total = (long long)rx1 * ry1, K = (long long)ry * n;
	for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
		const int a = int(e / ry1), c = int(e % ry1);
		double s = 0.0;
		for (long long k = 0; k < K; ++k) s += T[k * rx1 + a] * y[k * ry1 + c];
		M[e] = s;
	}
}

__global__ void k_zip_result(const double* M, double* out) { *out = M[0]; }

unsigned blocks_for(long long n) { return unsigned(n <= 0 ? 1 : (n + 255) / 256 > 1024 ? 1024 : (n + 255) / 256); }

bool is_device_pointer(const void* p, int& device) {
	cudaPointerAttributes a;
	if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
		cudaGetLastError();
		return false;
	}
	device = a.device;
	return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

int fail(int code, const std::string& msg) {
	xtt::set_last_error(msg);
	return code;
}

}  // namespace

extern "C" int xtt_dot_noalloc(int64_t order, const int64_t* dims, const int64_t* x_ranks, const double* x_cores,
                               const int64_t* y_ranks, const double* y_cores, double* result, void* stream) {
	if (!dims || !x_ranks || !y_ranks || !x_cores || !y_cores || !result)
		return fail(XTT_ERR_ARGUMENT, "xtt_dot_noalloc: NULL argument");
	if (order < 1) return fail(XTT_ERR_ARGUMENT, "xtt_dot_noalloc: order must be positive");
	if (x_ranks[0] != 1 || x_ranks[order] != 1 || y_ranks[0] != 1 || y_ranks[order] != 1)
		return fail(XTT_ERR_ARGUMENT, "xtt_dot_noalloc: boundary ranks must be 1");
	for (int64_t k = 0; k < order; ++k) {
		if (dims[k] < 1) return fail(XTT_ERR_ARGUMENT, "xtt_dot_noalloc: dimension 0 is not valid");
		if (dims[k] > kNoAllocMaxDim)
			return fail(XTT_ERR_CAPACITY, "xtt_dot_noalloc: mode size " + std::to_string(dims[k]) + " exceeds the limit " +
			                                  std::to_string(kNoAllocMaxDim));
	}
	for (int64_t k = 0; k <= order; ++k) {
		if (x_ranks[k] < 1 || y_ranks[k] < 1) return fail(XTT_ERR_ARGUMENT, "xtt_dot_noalloc: rank 0 is not valid");
		if (x_ranks[k] > kNoAllocMaxRank || y_ranks[k] > kNoAllocMaxRank)
			return fail(XTT_ERR_CAPACITY, "xtt_dot_noalloc: rank exceeds the limit " + std::to_string(kNoAllocMaxRank));
	}
	int dx = -1, dy = -1, dr = -1;
	if (!is_device_pointer(x_cores, dx) || !is_device_pointer(y_cores, dy) || !is_device_pointer(result, dr))
		return fail(XTT_ERR_ARGUMENT, "xtt_dot_noalloc: cores and result must be device memory");
	if (dx != dy || dx != dr) return fail(XTT_ERR_ARGUMENT, "xtt_dot_noalloc: pointers on different devices");
	if (dx < 0 || dx >= kMaxDevices) return fail(XTT_ERR_CAPACITY, "xtt_dot_noalloc: device index out of range");
	int current = -1;
	if (cudaGetDevice(&current) != cudaSuccess || current != dx)
		return fail(XTT_ERR_ARGUMENT, "xtt_dot_noalloc: the pointers' device must be the current device");
	cudaError_t err;
	double* base = scratch_on(dx, err);
	if (!base) return fail(XTT_ERR_CUDA, std::string("xtt_dot_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(err));
	double* M0 = base;
	double* M1 = base + kZipM;
	double* T = base + 2 * kZipM;
	cudaStream_t s = static_cast<cudaStream_t>(stream);
	// clear an error an earlier, unrelated call left behind, so that the check after the
	// launches reports this call's own launch errors only
	cudaGetLastError();
	k_zip_start<<<1, 1, 0, s>>>(M0);
	const double* xc = x_cores;
	const double* yc = y_cores;
	for (int64_t k = 0; k < order; ++k) {
		const int rx = int(x_ranks[k]), rx1 = int(x_ranks[k + 1]), ry = int(y_ranks[k]), ry1 = int(y_ranks[k + 1]);
		const int n = int(dims[k]);
		k_zip_left<<<blocks_for((long long)ry * n * rx1), 256, 0, s>>>(M0, xc, T, rx, ry, n, rx1);
		k_zip_right<<<blocks_for((long long)rx1 * ry1), 256, 0, s>>>(T, yc, M1, ry, n, rx1, ry1);
		double* t = M0;
		M0 = M1;
		M1 = t;
		xc += (long long)rx * n * rx1;
		yc += (long long)ry * n * ry1;
	}
	k_zip_result<<<1, 1, 0, s>>>(M0, result);
	err = cudaGetLastError();
	if (err != cudaSuccess) return fail(XTT_ERR_CUDA, std::string("xtt_dot_noalloc: ") + cudaGetErrorString(err));
	xtt::set_last_error("");
	return XTT_OK;
}
