// Quad generator on the GPU (replaces triNeighbours / quadNodes / genQuads of
// src/quad_generator.cpp, used by Scene::generateQuads, src/scene.cpp:237-246): pairs triangles
// that share an edge into quads, the input format of quad setup.
//
//  qgEdgeInsert    directed edges of every tri into an open-addressing hash table; the value is
//                  the lowest tri index holding the edge (the reference's first insertion wins).
//  qgNeighbours    neighbour across edge j of tri t: the tri of the reversed edge, unless t.
//  qgQuadFlags     (t, e) creates a quad when its neighbour b > t lists t back and has a vertex not
//                  in t (two tris sharing two edges share all vertices and never pair); quad ids
//                  are the exclusive scan of the flags in (t, e) order: the reference's creation
//                  order (quadNodes walks tris in order and the lower index of a pair creates it).
//  qgQuadBuild     vertices {t[e], opposite, t[e+1], t[e+2]}, squareness (normalize(v) = v / |v|;
//                  NaN counts as 0), the tris' quad slots.
//  qgConflicts     quads sharing a tri conflict.
//  qgScore/Pick/   synchronous rounds of the greedy independent set: every undecided quad scores
//  qgApply         conflicts - squareness * square_weight over its undecided conflicts (the
//                  reference's score, genQuads :138-141); the candidates are the undecided quads
//                  with the lowest live conflict count (the heap's leading term), and candidates
//                  whose (score, index) is below that of every conflicting candidate are
//                  selected together and their conflicts removed. Picks start at the mesh's
//                  boundaries and low-degree spots and advance as the counts drop, as in the
//                  reference, so about as few tris stay unpaired.
//                  (The reference selects one quad at a time from a heap and re-scores after
//                  each, which is sequential; the oracle computes both.)
//  qgOutput        tris in order: the tri's selected quad, nothing for the second tri of a
//                  selected quad, otherwise the degenerate quad (a, b, c, c).

#include <cstdio>
#include <string>
#include <vector>

#include "lucid_common.cuh"
#include "lucid_kernels.h"

namespace lucid {

namespace {

constexpr unsigned long long kEmptyKey = ~0ull;
constexpr int kQgThreads = 256;

__device__ __forceinline__ unsigned long long edgeKey(int a, int b) {
	return (static_cast<unsigned long long>(uint32_t(a)) << 32) | uint32_t(b);
}

__device__ __forceinline__ uint32_t hashKey(unsigned long long k) {
	k ^= k >> 33;
	k *= 0xff51afd7ed558ccdull;
	k ^= k >> 33;
	k *= 0xc4ceb9fe1a85ec53ull;
	k ^= k >> 33;
	return uint32_t(k);
}

struct QgQuad {
	int tris[2];
	int verts[4];
	int conflicts[4];
	float squareness;
	unsigned long long order; // (orderable score << 32) | quad index
};

__global__ void qgValidate(const int32_t* tris, int n3, int nv, int* bad) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i < n3 && (tris[i] < 0 || tris[i] >= nv))
		atomicExch(bad, 1);
}

__global__ void qgEdgeInsert(const int32_t* tris, int nt, unsigned long long* keys, int* vals, uint32_t mask) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= nt * 3)
		return;
	const int t = i / 3, j = i - t * 3;
	const unsigned long long k = edgeKey(tris[t * 3 + j], tris[t * 3 + (j == 2 ? 0 : j + 1)]);
	uint32_t slot = hashKey(k) & mask;
	for(uint32_t probe = 0; probe <= mask; probe++) { // the table is twice the edge count
		const unsigned long long prev = atomicCAS(&keys[slot], kEmptyKey, k);
		if(prev == kEmptyKey || prev == k) {
			atomicMin(&vals[slot], t);
			return;
		}
		slot = (slot + 1) & mask;
	}
}

__device__ __forceinline__ int edgeLookup(const unsigned long long* keys, const int* vals, uint32_t mask,
										  unsigned long long k) {
	uint32_t slot = hashKey(k) & mask;
	for(uint32_t probe = 0; probe <= mask; probe++) {
		const unsigned long long cur = keys[slot];
		if(cur == k)
			return vals[slot];
		if(cur == kEmptyKey)
			return -1;
		slot = (slot + 1) & mask;
	}
	return -1;
}

__global__ void qgNeighbours(const int32_t* tris, int nt, const unsigned long long* keys, const int* vals,
							 uint32_t mask, int* nb) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= nt * 3)
		return;
	const int t = i / 3, j = i - t * 3;
	const int v = edgeLookup(keys, vals, mask, edgeKey(tris[t * 3 + (j == 2 ? 0 : j + 1)], tris[t * 3 + j]));
	nb[i] = (v >= 0 && v != t) ? v : -1;
}

__device__ __forceinline__ int oppositeVertex(const int32_t* tris, int t, int b) {
	const int a0 = tris[t * 3], a1 = tris[t * 3 + 1], a2 = tris[t * 3 + 2];
	for(int k = 0; k < 3; k++) {
		const int v = tris[b * 3 + k];
		if(v != a0 && v != a1 && v != a2)
			return v;
	}
	return -1;
}

__device__ __forceinline__ int findTri(const int* nb, int b, int t) {
	for(int k = 0; k < 3; k++)
		if(nb[b * 3 + k] == t)
			return k;
	return -1;
}

__global__ void qgQuadFlags(const int32_t* tris, int nt, const int* nb, uint32_t* flags) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= nt * 3)
		return;
	const int t = i / 3;
	const int b = nb[i];
	flags[i] = (b > t && findTri(nb, b, t) >= 0 && oppositeVertex(tris, t, b) >= 0) ? 1u : 0u;
}

__device__ __forceinline__ F3 normalize3(F3 v) {
	const float l = sqrtf(dot3(v, v));
	return f3(v.x / l, v.y / l, v.z / l);
}

__global__ void qgQuadBuild(const float* positions, const int32_t* tris, int nt, const int* nb,
							const uint32_t* flags, const uint32_t* ids, QgQuad* quads, int* tri_quads) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= nt * 3 || !flags[i])
		return;
	const int t = i / 3, e = i - t * 3, b = nb[i];
	const int q = int(ids[i]);
	QgQuad qd;
	qd.tris[0] = t, qd.tris[1] = b;
	qd.verts[0] = tris[t * 3 + e];
	qd.verts[1] = oppositeVertex(tris, t, b);
	qd.verts[2] = tris[t * 3 + (e + 1) % 3];
	qd.verts[3] = tris[t * 3 + (e + 2) % 3];
	for(int k = 0; k < 4; k++)
		qd.conflicts[k] = -1;
	F3 c[4], ed[4];
	for(int k = 0; k < 4; k++)
		c[k] = xyz4(positions + size_t(qd.verts[k]) * 3);
	for(int k = 0; k < 4; k++)
		ed[k] = normalize3(c[(k + 1) & 3] - c[k]);
	float out = 0.0f;
	for(int k = 0; k < 4; k++)
		out += fabsf(dot3(ed[k], ed[(k + 1) & 3]));
	const float sq = (4.0f - out) * 0.25f;
	qd.squareness = sq == sq ? sq : 0.0f;
	qd.order = 0ull;
	quads[q] = qd;
	tri_quads[i] = q;
	tri_quads[b * 3 + findTri(nb, b, t)] = q;
}

__global__ void qgConflicts(QgQuad* quads, int nq, const int* tri_quads) {
	const int q = blockIdx.x * blockDim.x + threadIdx.x;
	if(q >= nq)
		return;
	QgQuad& qd = quads[q];
	int n = 0;
	for(int s = 0; s < 2; s++)
		for(int k = 0; k < 3; k++) {
			const int o = tri_quads[qd.tris[s] * 3 + k];
			if(o == -1 || o == q)
				continue;
			bool seen = false;
			for(int m = 0; m < n; m++)
				seen |= qd.conflicts[m] == o;
			if(!seen && n < 4)
				qd.conflicts[n++] = o;
		}
}

// state: 0 undecided, 1 removed, 2 selected. One round: the score of every undecided quad from
// its undecided conflicts, as an order key (orderable score bits << 32 | index), its live conflict
// count and the round's lowest count.
__global__ void qgScore(QgQuad* quads, int nq, const uint8_t* state, float square_weight, uint8_t* live_deg,
						int* min_deg) {
	const int q = blockIdx.x * blockDim.x + threadIdx.x;
	if(q >= nq || state[q] != 0)
		return;
	QgQuad& qd = quads[q];
	int live = 0;
	for(int k = 0; k < 4; k++)
		live += qd.conflicts[k] != -1 && state[qd.conflicts[k]] == 0;
	live_deg[q] = uint8_t(live);
	atomicMin(min_deg, live);
	float score = float(live) - qd.squareness * square_weight;
	if(score == 0.0f)
		score = 0.0f; // one zero
	const uint32_t u = fbits(score);
	const uint32_t ord = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
	qd.order = (static_cast<unsigned long long>(ord) << 32) | uint32_t(q);
}

// candidates: the undecided quads of the lowest live conflict count; a candidate below every
// conflicting candidate in the order is picked (two picked quads never conflict)
__global__ void qgPick(const QgQuad* quads, int nq, const uint8_t* state, const uint8_t* live_deg,
					   const int* min_deg, uint8_t* picked) {
	const int q = blockIdx.x * blockDim.x + threadIdx.x;
	if(q >= nq)
		return;
	const int md = *min_deg;
	auto candidate = [&](int x) { return state[x] == 0 && int(live_deg[x]) == md; };
	bool pick = candidate(q);
	if(pick) {
		const QgQuad& qd = quads[q];
		for(int k = 0; k < 4; k++) {
			const int c = qd.conflicts[k];
			if(c != -1 && candidate(c) && !(qd.order < quads[c].order))
				pick = false;
		}
	}
	picked[q] = pick ? 1 : 0;
}

__global__ void qgApply(const QgQuad* quads, int nq, uint8_t* state, const uint8_t* picked, int* undecided) {
	const int q = blockIdx.x * blockDim.x + threadIdx.x;
	if(q >= nq || !picked[q])
		return;
	state[q] = 2;
	for(int k = 0; k < 4; k++)
		if(quads[q].conflicts[k] != -1)
			state[quads[q].conflicts[k]] = 1;
}

__global__ void qgCountUndecided(const uint8_t* state, int nq, int* undecided) {
	const int q = blockIdx.x * blockDim.x + threadIdx.x;
	const bool u = q < nq && state[q] == 0;
	const int n = __syncthreads_count(u);
	if(threadIdx.x == 0 && n)
		atomicAdd(undecided, n);
}

__global__ void qgFillOnes(uint32_t* v, int n) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i < n)
		v[i] = 1u;
}

__global__ void qgSecondTris(const QgQuad* quads, int nq, const uint8_t* state, uint32_t* emit) {
	const int q = blockIdx.x * blockDim.x + threadIdx.x;
	if(q < nq && state[q] == 2)
		emit[quads[q].tris[1]] = 0u;
}

__global__ void qgOutput(const int32_t* tris, int nt, const QgQuad* quads, const int* tri_quads, const uint8_t* state,
						 const uint32_t* emit, const uint32_t* pos, uint32_t* out, uint32_t* degenerate) {
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if(t >= nt || !emit[t])
		return;
	int sel = -1;
	for(int k = 0; k < 3; k++) {
		const int q = tri_quads[t * 3 + k];
		if(q != -1 && state[q] == 2) {
			sel = q;
			break;
		}
	}
	uint4 o;
	if(sel == -1) {
		o = make_uint4(uint32_t(tris[t * 3]), uint32_t(tris[t * 3 + 1]), uint32_t(tris[t * 3 + 2]),
					   uint32_t(tris[t * 3 + 2]));
		atomicAdd(degenerate, 1u);
	} else {
		const QgQuad& qd = quads[sel];
		o = make_uint4(uint32_t(qd.verts[0]), uint32_t(qd.verts[1]), uint32_t(qd.verts[2]), uint32_t(qd.verts[3]));
	}
	reinterpret_cast<uint4*>(out)[pos[t]] = o;
}

// Exclusive scan of n u32 values (block sums, then their scan in one CTA, then the offsets).
constexpr int kScanBlock = 1024;

__global__ void scanBlocks(const uint32_t* in, uint32_t* out, uint32_t* sums, int n) {
	__shared__ uint32_t s_scan[kScanBlock / 32 + 1];
	const int i = blockIdx.x * kScanBlock + threadIdx.x;
	const uint32_t v = i < n ? in[i] : 0u;
	uint32_t total;
	const uint32_t ex = blockExclusiveScan(v, s_scan, &total);
	if(i < n)
		out[i] = ex;
	if(threadIdx.x == 0)
		sums[blockIdx.x] = total;
}

__global__ void scanSums(uint32_t* sums, int nblocks, uint32_t* total_out) {
	__shared__ uint32_t s_scan[kScanBlock / 32 + 1];
	uint32_t carry = 0;
	for(int base = 0; base < nblocks; base += kScanBlock) {
		const int i = base + threadIdx.x;
		const uint32_t v = i < nblocks ? sums[i] : 0u;
		uint32_t total;
		const uint32_t ex = blockExclusiveScan(v, s_scan, &total);
		if(i < nblocks)
			sums[i] = carry + ex;
		carry += total;
	}
	if(threadIdx.x == 0)
		*total_out = carry;
}

__global__ void scanAdd(uint32_t* out, const uint32_t* sums, int n) {
	const int i = blockIdx.x * kScanBlock + threadIdx.x;
	if(i < n)
		out[i] += sums[blockIdx.x];
}

} // namespace

// Exclusive scan of `in` into `out` (not aliased); the sum goes to *total (device).
static cudaError_t exclusiveScan(const uint32_t* in, uint32_t* out, uint32_t* sums, uint32_t* total, int n,
								 cudaStream_t s) {
	const int nb = (n + kScanBlock - 1) / kScanBlock;
	if(nb == 0)
		return cudaMemsetAsync(total, 0, 4, s);
	scanBlocks<<<nb, kScanBlock, 0, s>>>(in, out, sums, n);
	scanSums<<<1, kScanBlock, 0, s>>>(sums, nb, total);
	scanAdd<<<nb, kScanBlock, 0, s>>>(out, sums, n);
	return cudaGetLastError();
}

int quadGenerate(const float* positions, int num_verts, const int32_t* tris, int num_tris, float square_weight,
				 uint32_t* out_quads, int* out_num_quads, int* out_num_degenerate, cudaStream_t s, std::string& err) {
	*out_num_quads = 0;
	if(out_num_degenerate)
		*out_num_degenerate = 0;
	if(num_tris == 0)
		return 0;
	const int n3 = num_tris * 3;
	uint32_t tsize = 2;
	while(tsize < uint32_t(n3) * 2u)
		tsize <<= 1;
	const uint32_t mask = tsize - 1;
	const int nblk = (n3 + kScanBlock - 1) / kScanBlock + 1;
	// scratch
	std::vector<void*> allocs;
	auto alloc = [&](size_t bytes) -> void* {
		void* p = nullptr;
		if(cudaMalloc(&p, bytes < 16 ? 16 : bytes) != cudaSuccess) {
			cudaGetLastError();
			return nullptr;
		}
		allocs.push_back(p);
		return p;
	};
	auto cleanup = [&]() {
		cudaStreamSynchronize(s);
		for(void* p : allocs)
			cudaFree(p);
	};
	unsigned long long* keys = (unsigned long long*)alloc(size_t(tsize) * 8);
	int* vals = (int*)alloc(size_t(tsize) * 4);
	int* nb = (int*)alloc(size_t(n3) * 4);
	uint32_t* flags = (uint32_t*)alloc(size_t(n3) * 4);
	uint32_t* ids = (uint32_t*)alloc(size_t(n3) * 4);
	uint32_t* sums = (uint32_t*)alloc(size_t(nblk) * 4);
	int* tri_quads = (int*)alloc(size_t(n3) * 4);
	uint32_t* emit = (uint32_t*)alloc(size_t(num_tris) * 4);
	uint32_t* pos = (uint32_t*)alloc(size_t(num_tris) * 4);
	int* counters = (int*)alloc(16); // [0] bad index, [1] undecided, [2] quads, [3] degenerate
	if(!keys || !vals || !nb || !flags || !ids || !sums || !tri_quads || !emit || !pos || !counters) {
		cleanup();
		err = "quad generator: out of device memory";
		return 2;
	}
	const int g3 = (n3 + kQgThreads - 1) / kQgThreads, gt = (num_tris + kQgThreads - 1) / kQgThreads;
	cudaMemsetAsync(counters, 0, 16, s);
	qgValidate<<<g3, kQgThreads, 0, s>>>(tris, n3, num_verts, counters);
	int host[4] = {0, 0, 0, 0};
	cudaMemcpyAsync(host, counters, 16, cudaMemcpyDeviceToHost, s);
	cudaError_t ce = cudaStreamSynchronize(s);
	if(ce != cudaSuccess || host[0]) {
		cleanup();
		err = ce != cudaSuccess ? std::string("quad generator: ") + cudaGetErrorString(ce)
								: "quad generator: vertex index out of range";
		return ce != cudaSuccess ? 3 : 1;
	}
	cudaMemsetAsync(keys, 0xff, size_t(tsize) * 8, s);
	cudaMemsetAsync(vals, 0x7f, size_t(tsize) * 4, s);
	qgEdgeInsert<<<g3, kQgThreads, 0, s>>>(tris, num_tris, keys, vals, mask);
	qgNeighbours<<<g3, kQgThreads, 0, s>>>(tris, num_tris, keys, vals, mask, nb);
	qgQuadFlags<<<g3, kQgThreads, 0, s>>>(tris, num_tris, nb, flags);
	exclusiveScan(flags, ids, sums, reinterpret_cast<uint32_t*>(counters + 2), n3, s);
	cudaMemcpyAsync(host, counters, 16, cudaMemcpyDeviceToHost, s);
	if((ce = cudaStreamSynchronize(s)) != cudaSuccess) {
		cleanup();
		err = std::string("quad generator: ") + cudaGetErrorString(ce);
		return 3;
	}
	const int nq = host[2];
	QgQuad* quads = (QgQuad*)alloc(size_t(nq) * sizeof(QgQuad));
	uint8_t* state = (uint8_t*)alloc(size_t(nq));
	uint8_t* picked = (uint8_t*)alloc(size_t(nq));
	uint8_t* live_deg = (uint8_t*)alloc(size_t(nq));
	if(!quads || !state || !picked || !live_deg) {
		cleanup();
		err = "quad generator: out of device memory";
		return 2;
	}
	cudaMemsetAsync(tri_quads, 0xff, size_t(n3) * 4, s);
	cudaMemsetAsync(state, 0, size_t(nq), s);
	qgQuadBuild<<<g3, kQgThreads, 0, s>>>(positions, tris, num_tris, nb, flags, ids, quads, tri_quads);
	const int gq = (nq + kQgThreads - 1) / kQgThreads;
	if(nq > 0) {
		qgConflicts<<<gq, kQgThreads, 0, s>>>(quads, nq, tri_quads);
		// rounds until every quad is decided (each round picks at least the first undecided quad
		// of the order, so nq rounds bound it); the host checks after every 16 rounds (rounds
		// after the last decision change nothing)
		for(int round = 0; round <= nq; round += 16) {
			for(int k = 0; k < 16; k++) {
				cudaMemsetAsync(counters, 0x7f, 4, s); // [0] lowest live conflict count
				qgScore<<<gq, kQgThreads, 0, s>>>(quads, nq, state, square_weight, live_deg, counters);
				qgPick<<<gq, kQgThreads, 0, s>>>(quads, nq, state, live_deg, counters, picked);
				qgApply<<<gq, kQgThreads, 0, s>>>(quads, nq, state, picked, counters + 1);
			}
			cudaMemsetAsync(counters + 1, 0, 4, s); // [1] undecided
			qgCountUndecided<<<gq, kQgThreads, 0, s>>>(state, nq, counters + 1);
			int undecided = 0;
			cudaMemcpyAsync(&undecided, counters + 1, 4, cudaMemcpyDeviceToHost, s);
			if((ce = cudaStreamSynchronize(s)) != cudaSuccess)
				break;
			if(undecided == 0)
				break;
		}
	}
	// output positions: every tri but the second tri of a selected quad
	qgFillOnes<<<gt, kQgThreads, 0, s>>>(emit, num_tris);
	if(nq > 0)
		qgSecondTris<<<gq, kQgThreads, 0, s>>>(quads, nq, state, emit);
	exclusiveScan(emit, pos, sums, reinterpret_cast<uint32_t*>(counters + 2), num_tris, s);
	cudaMemsetAsync(counters + 3, 0, 4, s);
	qgOutput<<<gt, kQgThreads, 0, s>>>(tris, num_tris, quads, tri_quads, state, emit, pos, out_quads,
										reinterpret_cast<uint32_t*>(counters + 3));
	cudaMemcpyAsync(host, counters, 16, cudaMemcpyDeviceToHost, s);
	ce = cudaStreamSynchronize(s);
	if(ce == cudaSuccess)
		ce = cudaGetLastError();
	cleanup();
	if(ce != cudaSuccess) {
		err = std::string("quad generator: ") + cudaGetErrorString(ce);
		return 3;
	}
	*out_num_quads = host[2];
	if(out_num_degenerate)
		*out_num_degenerate = host[3];
	return 0;
}

} // namespace lucid
