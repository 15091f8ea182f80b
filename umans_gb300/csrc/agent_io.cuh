// AgentData exchange: packing and unpacking agent records
//
// Device code of the step engine, part of engine.cu's translation unit:
// included once, from engine.cu, after DevState; uses its helpers.
#pragma once

namespace umans {

// The AgentData records (28 bytes: id, position, velocity, viewing
// direction) move through shared memory, so that the block's stretch of
// records is read or written as consecutive 4-byte words: coalesced, also
// when the buffer is page-locked host memory that the kernel accesses
// directly.
constexpr int PACK_BLOCK = 256, REC_WORDS = (int)(sizeof(AgentRecord) / 4);
static_assert(sizeof(AgentRecord) == 28, "AgentData layout");

// GetAgentPositions (APIFunctions.cpp:88-115): the records of slots [0, n)
__global__ void __launch_bounds__(PACK_BLOCK) k_pack(DevState S, AgentRecord* dst)
{
	__shared__ uint32_t w[PACK_BLOCK * REC_WORDS];
	const int i0 = blockIdx.x * PACK_BLOCK, i = i0 + threadIdx.x;
	const int cnt = min(PACK_BLOCK, S.n - i0);
	if (i < S.n) {
		const float2 p = S.pos[i], v = S.vel[i], vw = S.view[i];
		uint32_t* r = w + threadIdx.x * REC_WORDS;
		r[0] = (uint32_t)S.id[i];
		r[1] = __float_as_uint(p.x); r[2] = __float_as_uint(p.y);
		r[3] = __float_as_uint(v.x); r[4] = __float_as_uint(v.y);
		r[5] = __float_as_uint(vw.x); r[6] = __float_as_uint(vw.y);
	}
	__syncthreads();
	uint32_t* out = reinterpret_cast<uint32_t*>(dst) + (size_t)i0 * REC_WORDS;
	for (int k = threadIdx.x; k < cnt * REC_WORDS; k += PACK_BLOCK) out[k] = w[k];
}

// SetAgentPositions (APIFunctions.cpp:117-137): Agent::setPosition and
// Agent::setVelocity_ExternalApplication for every listed id that exists
__global__ void __launch_bounds__(PACK_BLOCK) k_unpack(DevState S, const AgentRecord* src, int m)
{
	__shared__ uint32_t w[PACK_BLOCK * REC_WORDS];
	const int k0 = blockIdx.x * PACK_BLOCK, k = k0 + threadIdx.x;
	const int cnt = min(PACK_BLOCK, m - k0);
	const uint32_t* in = reinterpret_cast<const uint32_t*>(src) + (size_t)k0 * REC_WORDS;
	for (int j = threadIdx.x; j < cnt * REC_WORDS; j += PACK_BLOCK) w[j] = in[j];
	__syncthreads();
	if (k >= m) return;
	const uint32_t* r = w + threadIdx.x * REC_WORDS;
	const int id = (int)r[0];
	if (id < 0 || id >= S.id_bound) return;
	const int i = S.slot_of_id[id];
	if (i < 0) return;
	S.pos[i] = V(__uint_as_float(r[1]), __uint_as_float(r[2]));
	S.vel[i] = V(__uint_as_float(r[3]), __uint_as_float(r[4]));
	S.vwf[i] = V(__uint_as_float(r[3]), __uint_as_float(r[4]));
	S.view[i] = V(__uint_as_float(r[5]), __uint_as_float(r[6]));
}

}  // namespace umans
