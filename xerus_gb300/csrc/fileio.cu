// xerus's binary file format for TTTensor / TTOperator (misc::save_to_file /
// load_from_file, include/xerus/misc/fileIO.h:103-162), so device tensors can be
// checkpointed to and resumed from files xerus itself reads and writes.
//
// Layout (little-endian, size_t = u64, bool = 1 byte), as written by the
// reference's stream writers:
//   "Xerus xerus::TTNetwork<false|true> datafile.\nFormat: Binary\n"
//   TTNetwork (src/xerus/ttNetwork.cpp:1454-1468): u64 1, bool canonicalized, u64 corePosition
//   TensorNetwork (src/xerus/tensorNetwork.cpp:1429-1466): u64 1, dimensions (u64 count + u64
//     each; an operator lists the d row then the d column dimensions), per dimension the
//     external link (u64 node, u64 index position, u64 dimension), u64 node count (d + 2:
//     a virtual rank-1 node on each side), per node its links (u64 count, then bool
//     external, u64 other node (max for external), u64 index position, u64 dimension)
//   per node its Tensor (src/xerus/tensor.cpp:1781-1802): u64 1, dimensions, u64
//     representation (1 dense: values; 2 sparse: u64 count, then (u64 index, double) pairs)
// Host code only: the cores move to and from the device through the tensor API.
#include <cstdint>
#include <cstring>
#include <fstream>
#include <iterator>
#include <limits>
#include <string>
#include <vector>

#include "engine.cuh"

namespace xtt {

namespace {

struct Writer {
	std::vector<uint8_t> out;
	void raw(const void* p, size_t n) {
		const uint8_t* b = static_cast<const uint8_t*>(p);
		out.insert(out.end(), b, b + n);
	}
	void u64(uint64_t v) { raw(&v, 8); }
	void boolean(bool v) {
		const uint8_t b = v ? 1 : 0;
		raw(&b, 1);
	}
	void f64(double v) { raw(&v, 8); }
};

struct Reader {
	const uint8_t* p;
	size_t n, at = 0;
	void need(size_t k) {
		if (at + k > n) throw Error(XTT_ERR_ARGUMENT, "unexpected end of xerus data file");
	}
	uint64_t u64() {
		need(8);
		uint64_t v;
		std::memcpy(&v, p + at, 8);
		at += 8;
		return v;
	}
	bool boolean() {
		need(1);
		return p[at++] != 0;
	}
	double f64() {
		need(8);
		double v;
		std::memcpy(&v, p + at, 8);
		at += 8;
		return v;
	}
};

const char* type_name(bool op) { return op ? "xerus::TTNetwork<true>" : "xerus::TTNetwork<false>"; }

}  // namespace

std::vector<uint8_t> tt_file_encode(bool op, const std::vector<int64_t>& dims, const std::vector<int64_t>& ranks,
                                    const double* cores, bool canonicalized, int64_t core_position) {
	const int d = int(dims.size());
	XTT_REQUIRE(int(ranks.size()) == d + 1 && d >= 1, "dims and ranks do not describe a TT");
	const uint64_t npos = std::numeric_limits<uint64_t>::max();
	const int order = op ? 2 : 1;  // external indices per component
	Writer w;
	const std::string header = std::string("Xerus ") + type_name(op) + " datafile.\nFormat: Binary\n";
	w.raw(header.data(), header.size());
	w.u64(1);
	w.boolean(canonicalized);
	w.u64(uint64_t(core_position));
	w.u64(1);
	w.u64(uint64_t(order * d));
	for (int r = 0; r < order; ++r)
		for (int k = 0; k < d; ++k) w.u64(uint64_t(dims[k]));
	for (int r = 0; r < order; ++r)
		for (int k = 0; k < d; ++k) {
			w.u64(uint64_t(k + 1));
			w.u64(uint64_t(1 + r));
			w.u64(uint64_t(dims[k]));
		}
	w.u64(uint64_t(d + 2));
	const uint64_t right_pos = uint64_t(order + 1);  // index position of a component's right bond
	// node 0: the left virtual node
	w.u64(1);
	w.boolean(false);
	w.u64(1);
	w.u64(0);
	w.u64(1);
	for (int k = 0; k < d; ++k) {
		w.u64(uint64_t(order + 2));
		w.boolean(false);  // left bond
		w.u64(uint64_t(k));
		w.u64(k == 0 ? 0 : right_pos);
		w.u64(uint64_t(ranks[k]));
		for (int r = 0; r < order; ++r) {  // external indices
			w.boolean(true);
			w.u64(npos);
			w.u64(uint64_t(r * d + k));
			w.u64(uint64_t(dims[k]));
		}
		w.boolean(false);  // right bond
		w.u64(uint64_t(k + 2));
		w.u64(0);
		w.u64(uint64_t(ranks[k + 1]));
	}
	// node d+1: the right virtual node
	w.u64(1);
	w.boolean(false);
	w.u64(uint64_t(d));
	w.u64(right_pos);
	w.u64(1);
	// tensors: virtual [1] = 1, components dense
	auto unit = [&] {
		w.u64(1);
		w.u64(1);
		w.u64(1);
		w.u64(1);
		w.f64(1.0);
	};
	unit();
	size_t off = 0;
	for (int k = 0; k < d; ++k) {
		w.u64(1);
		w.u64(uint64_t(order + 2));
		w.u64(uint64_t(ranks[k]));
		for (int r = 0; r < order; ++r) w.u64(uint64_t(dims[k]));
		w.u64(uint64_t(ranks[k + 1]));
		w.u64(1);
		size_t cnt = size_t(ranks[k]) * size_t(ranks[k + 1]);
		for (int r = 0; r < order; ++r) cnt *= size_t(dims[k]);
		for (size_t i = 0; i < cnt; ++i) w.f64(cores[off + i]);
		off += cnt;
	}
	unit();
	return w.out;
}

TtFile tt_file_decode(const uint8_t* data, size_t size) {
	Reader r{data, size};
	// header: two lines
	size_t nl1 = 0;
	while (nl1 < size && data[nl1] != '\n') ++nl1;
	XTT_REQUIRE(nl1 < size, "not a xerus data file");
	const std::string first(reinterpret_cast<const char*>(data), nl1);
	TtFile f;
	if (first == std::string("Xerus ") + type_name(false) + " datafile.") f.op = false;
	else if (first == std::string("Xerus ") + type_name(true) + " datafile.") f.op = true;
	else throw Error(XTT_ERR_ARGUMENT, "not a xerus TTTensor / TTOperator data file: " + first);
	size_t nl2 = nl1 + 1;
	while (nl2 < size && data[nl2] != '\n') ++nl2;
	XTT_REQUIRE(nl2 < size, "truncated xerus data file header");
	const std::string second(reinterpret_cast<const char*>(data + nl1 + 1), nl2 - nl1 - 1);
	XTT_REQUIRE(second == "Format: Binary", "only the binary xerus format is supported");
	r.at = nl2 + 1;
	XTT_REQUIRE(r.u64() == 1, "unknown TTNetwork stream version");
	f.canonicalized = r.boolean();
	f.core_position = int64_t(r.u64());
	XTT_REQUIRE(r.u64() == 1, "unknown TensorNetwork stream version");
	const uint64_t nd = r.u64();
	const int order = f.op ? 2 : 1;
	XTT_REQUIRE(nd >= uint64_t(order) && nd % order == 0 && nd < (1u << 20), "inconsistent dimension count");
	const int d = int(nd / order);
	std::vector<uint64_t> alld(nd);
	for (auto& v : alld) v = r.u64();
	for (uint64_t i = 0; i < nd; ++i) {
		r.u64();
		r.u64();
		r.u64();
	}
	const uint64_t nn = r.u64();
	XTT_REQUIRE(nn == uint64_t(d + 2), "not a TT network (node count)");
	for (uint64_t k = 0; k < nn; ++k) {
		const uint64_t m = r.u64();
		XTT_REQUIRE(m < 64, "implausible link count");
		for (uint64_t l = 0; l < m; ++l) {
			r.boolean();
			r.u64();
			r.u64();
			r.u64();
		}
	}
	f.dims.assign(d, 0);
	f.ranks.assign(d + 1, 1);
	for (int k = 0; k < d; ++k) f.dims[k] = int64_t(alld[k]);
	for (uint64_t k = 0; k < nn; ++k) {
		XTT_REQUIRE(r.u64() == 1, "unknown Tensor stream version");
		const uint64_t td = r.u64();
		XTT_REQUIRE(td < 64, "implausible tensor order");
		std::vector<uint64_t> tdims(td);
		uint64_t cnt = 1;
		for (auto& v : tdims) {
			v = r.u64();
			cnt *= v;
		}
		const uint64_t rep = r.u64();
		std::vector<double> vals(cnt, 0.0);
		if (rep == 1) {
			r.need(cnt * 8);
			std::memcpy(vals.data(), data + r.at, cnt * 8);
			r.at += cnt * 8;
		} else {
			XTT_REQUIRE(rep == 2, "unknown tensor representation");
			const uint64_t ne = r.u64();
			for (uint64_t e = 0; e < ne; ++e) {
				const uint64_t idx = r.u64();
				const double v = r.f64();
				XTT_REQUIRE(idx < cnt, "sparse entry out of range");
				vals[idx] = v;
			}
		}
		if (k == 0 || k == nn - 1) continue;  // virtual nodes
		const int c = int(k) - 1;
		XTT_REQUIRE(td == uint64_t(order + 2), "component of the wrong order");
		for (int q = 0; q < order; ++q)
			XTT_REQUIRE(int64_t(tdims[1 + q]) == f.dims[c], "component dimension differs from the network's");
		XTT_REQUIRE(int64_t(tdims[0]) == f.ranks[c], "left rank differs from the neighbour's");
		f.ranks[c + 1] = int64_t(tdims[td - 1]);
		f.cores.insert(f.cores.end(), vals.begin(), vals.end());
	}
	XTT_REQUIRE(f.ranks[d] == 1, "last rank must be 1");
	XTT_REQUIRE(r.at == size, "trailing bytes after the TT data");
	return f;
}

std::vector<uint8_t> read_file(const std::string& path) {
	std::ifstream in(path, std::ios::binary);
	XTT_REQUIRE(in, "cannot open " + path);
	return std::vector<uint8_t>((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
}

void write_file(const std::string& path, const std::vector<uint8_t>& bytes) {
	std::ofstream out(path, std::ios::binary | std::ios::trunc);
	XTT_REQUIRE(out, "cannot open " + path + " for writing");
	out.write(reinterpret_cast<const char*>(bytes.data()), std::streamsize(bytes.size()));
	XTT_REQUIRE(out, "write to " + path + " failed");
}

}  // namespace xtt
