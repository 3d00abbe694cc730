/* nrc.cu -- the radiance cache: a small MLP that stands in for the photon-map
 * final gather of indirect light, trained online on the gather's own
 * estimates (no counterpart in the reference; the final gather it replaces is
 * shade_phong's diffuse rays + PhotonMap::radiance_est, src/shader.cc:154-187,
 * src/pmap.cc:143-178).
 *
 * Network: 9 inputs (position scaled to the scene box, normal, direction),
 * 12-band sin/cos encoding (216 features), 4 hidden layers of 64 ReLU units,
 * 3 linear outputs; relative L2 loss; Adam.  Weights are kept in FP32 (the
 * Adam master copy) and used as BF16 with FP32 accumulation: inference and
 * queries on the 5th-generation tensor cores (tcgen05.mma, a 128-sample tile
 * per MMA); the training step by warp-level MMAs (mma.sync m16n8k16: a warp
 * carries 16 samples through all five layers with the activations in
 * registers, the accumulator tile of one layer becoming the operand tile of
 * the next).
 *
 *   k_nrc_forward_tc<FWD_INFER>  inference: encode + 5 layers on the
 *                         5th-generation tensor cores (TMEM accumulators
 *                         and hidden operands, three tiles in flight per SM)
 *   k_nrc_forward_tc<FWD_QUERY>  the renderer's queries: the same, the output
 *                         weighted into the pixel's accumulator
 *   k_nrc_forward<FWD_TRAIN>  training forward (warp-level MMA): also stores
 *                         the layer inputs (BF16) and the loss gradient of
 *                         the outputs
 *   k_nrc_backward        dZ of layers 4..1 through the transposed weights,
 *                         bias gradients
 *   k_nrc_wgrad<L>        weight gradients dW = dZ^T H over the batch (MMA,
 *                         samples split over blocks, FP32 atomics)
 *   k_nrc_adam            Adam on the FP32 master, BF16 copies refreshed
 *
 * The CPU restatement (checker of these kernels) is oracle/nrc.py.
 */
#include <math.h>
#include <string.h>
#include <stdint.h>
#include <vector>
#include <mutex>
#include <string>
#include <cuda_bf16.h>
#include "sray_gpu.h"
#include "sray_rng.h"
#include "nrc.h"

namespace sray {

/* ---- parameter layout (packed FP32, the order of oracle/nrc.py) ---- */
enum {
	NRC_F = 216,            /* encoded features */
	NRC_FP = 224,           /* padded to 14 k-tiles of 16 */
	NRC_H = 64,
	NRC_O = 3,
	OFF_W1 = 0,
	OFF_B1 = OFF_W1 + NRC_H * NRC_F,
	OFF_W2 = OFF_B1 + NRC_H,
	OFF_B2 = OFF_W2 + NRC_H * NRC_H,
	OFF_W3 = OFF_B2 + NRC_H,
	OFF_B3 = OFF_W3 + NRC_H * NRC_H,
	OFF_W4 = OFF_B3 + NRC_H,
	OFF_B4 = OFF_W4 + NRC_H * NRC_H,
	OFF_W5 = OFF_B4 + NRC_H,
	OFF_B5 = OFF_W5 + NRC_O * NRC_H,
	NRC_NPARAM = OFF_B5 + NRC_O
};
static_assert(NRC_NPARAM == SRAY_NRC_PARAMS, "parameter count");

/* shared-memory row strides (bf16 elements), padded against bank conflicts */
enum { LD1 = 232, LDH = 72, LD5T = 24 };
#define NRC_FWD_THREADS 256   /* forward blocks: 8 warps share one copy of the weights in shared memory */

/* BF16 weight images in global memory, in the shared-memory layout:
 *   w1  [64][LD1]      (in 0..215, zero up to 231)
 *   w2-4 [64][LDH]     (out rows, in columns)
 *   w5  [8][LDH]       (rows 3..7 zero)
 *   w2t-w4t [64][LDH]  transposed (in rows, out columns), for the backward pass
 *   w5t [64][LD5T]     transposed, out columns 3..23 zero
 * plus the FP32 biases b1-b4 [64], b5 [8]. */
struct NrcDev {
	const __nv_bfloat16 *w1, *w2, *w3, *w4, *w5;
	const __nv_bfloat16 *w2t, *w3t, *w4t, *w5t;
	const float *bias;            /* 4 x 64 + 8 */
};

enum {
	IMG_W1 = 0,
	IMG_W2 = IMG_W1 + 64 * LD1,
	IMG_W3 = IMG_W2 + 64 * LDH,
	IMG_W4 = IMG_W3 + 64 * LDH,
	IMG_W5 = IMG_W4 + 64 * LDH,
	IMG_W2T = IMG_W5 + 8 * LDH,
	IMG_W3T = IMG_W2T + 64 * LDH,
	IMG_W4T = IMG_W3T + 64 * LDH,
	IMG_W5T = IMG_W4T + 64 * LDH,
	IMG_END = IMG_W5T + 64 * LD5T,
	FWD_SMEM_BF16 = IMG_W2T,                /* w1..w5 */
	BWD_SMEM_BF16 = IMG_END - IMG_W2T,      /* w2t..w5t */
	NRC_NBIAS = 4 * 64 + 8
};

/* ---- warp-level MMA tiles ---- */
__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
	asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
			: "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
			: "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
	__nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
	return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ float bf16_lo(uint32_t v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t v) { return __uint_as_float(v & 0xffff0000u); }

/* B operand of a k16 x n8 tile whose element (k, n) is M[n0 + n][k0 + k] of
 * a row-major shared matrix with row stride ld: two adjacent k per register */
__device__ __forceinline__ void load_b(const __nv_bfloat16 *M, int ld, int n0, int k0, int lane, uint32_t &b0, uint32_t &b1)
{
	int g = lane >> 2, t = lane & 3;
	const __nv_bfloat16 *p = M + (size_t)(n0 + g) * ld + k0 + 2 * t;
	b0 = *reinterpret_cast<const uint32_t *>(p);
	b1 = *reinterpret_cast<const uint32_t *>(p + 8);
}

/* a 16 x 64 activation block as accumulators: 8 n-tiles x 4 floats */
struct Acc64 {
	float d[8][4];
};

/* accumulators of a layer -> A operand tiles of the next (BF16): k-tile kt
 * is made of n-tiles 2kt and 2kt+1 */
__device__ __forceinline__ void acc_to_a(const Acc64 &z, uint32_t (&a)[4][4], bool relu)
{
	#pragma unroll
	for(int kt = 0; kt < 4; kt++) {
		const float *lo = z.d[2 * kt], *hi = z.d[2 * kt + 1];
		float v[8] = {lo[0], lo[1], lo[2], lo[3], hi[0], hi[1], hi[2], hi[3]};
		if(relu) {
			#pragma unroll
			for(int i = 0; i < 8; i++) v[i] = fmaxf(v[i], 0.0f);
		}
		a[kt][0] = pack_bf16(v[0], v[1]);
		a[kt][1] = pack_bf16(v[2], v[3]);
		a[kt][2] = pack_bf16(v[4], v[5]);
		a[kt][3] = pack_bf16(v[6], v[7]);
	}
}

/* 16 x 64 = A(16 x 64) W^T: W [64][LDH] (out, in) */
__device__ __forceinline__ void layer64(const uint32_t (&a)[4][4], const __nv_bfloat16 *W, const float *bias, int lane, Acc64 &z)
{
	int t = lane & 3;
	#pragma unroll
	for(int nt = 0; nt < 8; nt++) {
		float b0 = bias[nt * 8 + 2 * t], b1 = bias[nt * 8 + 2 * t + 1];
		z.d[nt][0] = b0; z.d[nt][1] = b1; z.d[nt][2] = b0; z.d[nt][3] = b1;
		#pragma unroll
		for(int kt = 0; kt < 4; kt++) {
			uint32_t w0, w1;
			load_b(W, LDH, nt * 8, kt * 16, lane, w0, w1);
			mma16816(z.d[nt], a[kt], w0, w1);
		}
	}
}

/* one encoded feature pair (sin, cos of pi 2^b x_v) for pair index p, 0 for padding */
__device__ __forceinline__ uint32_t feature_pair(const float *x, int p)
{
	if(p >= NRC_F / 2) return 0u;
	int v = p / 12, b = p - v * 12;
	float s, c;
	sincospif(x[v] * (float)(1 << b), &s, &c);
	return pack_bf16(s, c);
}

/* the A operand of k-tile kt of the encoded inputs, rows g and g + 8 */
__device__ __forceinline__ void encode_a(const float *xg, const float *xg8, int kt, int lane, uint32_t (&a)[4])
{
	int t = lane & 3;
	int p0 = kt * 8 + t, p1 = kt * 8 + 4 + t;
	a[0] = feature_pair(xg, p0);
	a[1] = feature_pair(xg8, p0);
	a[2] = feature_pair(xg, p1);
	a[3] = feature_pair(xg8, p1);
}

__device__ __forceinline__ void copy_to_shared(__nv_bfloat16 *dst, const __nv_bfloat16 *src, int n)
{
	const uint4 *s = reinterpret_cast<const uint4 *>(src);
	uint4 *d = reinterpret_cast<uint4 *>(dst);
	for(int i = threadIdx.x; i < n / 8; i += blockDim.x) d[i] = s[i];
}

/* Forward pass, a warp per 16 samples.  x: [n][9]; y: [n][3] (inference) or
 * unused.  TRAIN: t [n][3] targets; stores h0 [n16][NRC_FP] (encoded, BF16),
 * h1..h4 [n16][64] (BF16), dz5 [n16][16] (BF16 loss gradient of the
 * outputs), db5 partial sums and the loss. */
struct TrainBufs {
	__nv_bfloat16 *h[5];          /* h[0] encoded inputs, h[1..4] hidden */
	__nv_bfloat16 *dz[6];         /* dz[1..4] hidden, dz[5] outputs (16 wide) */
	float *grad;                  /* packed FP32 gradient */
	float *loss;
};

/* queries of the renderer: inputs x [n][9]; w[i] = weight rgb and the
 * accumulator slot; acc[slot] += w * max(y, 0); the count is read on the
 * device (n is the capacity) */
struct QueryOut {
	const int *count;
	const float4 *w;
	float4 *acc;
};

enum { FWD_INFER = 0, FWD_TRAIN = 1, FWD_QUERY = 2 };

template <int MODE>
__global__ void __launch_bounds__(NRC_FWD_THREADS) k_nrc_forward(NrcDev net, int n, const float *x, float *y, const float *tgt, TrainBufs tb,
		QueryOut qo)
{
	constexpr bool TRAIN = MODE == FWD_TRAIN;
	if(MODE == FWD_QUERY) {
		int c = *qo.count;
		n = c < n ? c : n;
	}
	extern __shared__ __align__(16) unsigned char smem_raw[];
	__nv_bfloat16 *sw = reinterpret_cast<__nv_bfloat16 *>(smem_raw);
	float *sb = reinterpret_cast<float *>(sw + FWD_SMEM_BF16);
	copy_to_shared(sw, net.w1, FWD_SMEM_BF16);
	for(int i = threadIdx.x; i < NRC_NBIAS; i += blockDim.x) sb[i] = net.bias[i];
	__syncthreads();
	const __nv_bfloat16 *W1 = sw + IMG_W1, *W2 = sw + IMG_W2, *W3 = sw + IMG_W3, *W4 = sw + IMG_W4, *W5 = sw + IMG_W5;
	int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	int g = lane >> 2, t = lane & 3;
	int ntiles = (n + 15) >> 4;
	float loss = 0.0f;
	float db5[2] = {0.0f, 0.0f};
	const int wpb = NRC_FWD_THREADS / 32;
	for(int tile = blockIdx.x * wpb + warp; tile < ntiles; tile += gridDim.x * wpb) {
		int r0 = tile * 16 + g, r1 = r0 + 8;
		float xg[9], xg8[9];
		#pragma unroll
		for(int k = 0; k < 9; k++) {
			xg[k] = r0 < n ? x[(size_t)r0 * 9 + k] : 0.0f;
			xg8[k] = r1 < n ? x[(size_t)r1 * 9 + k] : 0.0f;
		}
		/* layer 1: 14 k-tiles of encoded features */
		Acc64 z;
		#pragma unroll
		for(int nt = 0; nt < 8; nt++) {
			float b0 = sb[nt * 8 + 2 * t], b1 = sb[nt * 8 + 2 * t + 1];
			z.d[nt][0] = b0; z.d[nt][1] = b1; z.d[nt][2] = b0; z.d[nt][3] = b1;
		}
		for(int kt = 0; kt < NRC_FP / 16; kt++) {
			uint32_t a[4];
			encode_a(xg, xg8, kt, lane, a);
			if(TRAIN) {
				__nv_bfloat16 *h0 = tb.h[0];
				uint32_t *p0 = reinterpret_cast<uint32_t *>(h0 + (size_t)r0 * NRC_FP + kt * 16 + 2 * t);
				uint32_t *p1 = reinterpret_cast<uint32_t *>(h0 + (size_t)r1 * NRC_FP + kt * 16 + 2 * t);
				p0[0] = a[0]; p1[0] = a[1]; p0[4] = a[2]; p1[4] = a[3];
			}
			#pragma unroll
			for(int nt = 0; nt < 8; nt++) {
				uint32_t w0, w1;
				load_b(W1, LD1, nt * 8, kt * 16, lane, w0, w1);
				mma16816(z.d[nt], a, w0, w1);
			}
		}
		uint32_t a[4][4];
		const __nv_bfloat16 *Ws[3] = {W2, W3, W4};
		#pragma unroll
		for(int l = 0; l < 3; l++) {
			acc_to_a(z, a, true);
			if(TRAIN) {
				/* h_{l+1}: the BF16 input of layer l + 2 */
				__nv_bfloat16 *h = tb.h[l + 1];
				#pragma unroll
				for(int kt = 0; kt < 4; kt++) {
					uint32_t *p0 = reinterpret_cast<uint32_t *>(h + (size_t)r0 * 64 + kt * 16 + 2 * t);
					uint32_t *p1 = reinterpret_cast<uint32_t *>(h + (size_t)r1 * 64 + kt * 16 + 2 * t);
					p0[0] = a[kt][0]; p1[0] = a[kt][1]; p0[4] = a[kt][2]; p1[4] = a[kt][3];
				}
			}
			layer64(a, Ws[l], sb + 64 * (l + 1), lane, z);
		}
		acc_to_a(z, a, true);
		if(TRAIN) {
			__nv_bfloat16 *h = tb.h[4];
			#pragma unroll
			for(int kt = 0; kt < 4; kt++) {
				uint32_t *p0 = reinterpret_cast<uint32_t *>(h + (size_t)r0 * 64 + kt * 16 + 2 * t);
				uint32_t *p1 = reinterpret_cast<uint32_t *>(h + (size_t)r1 * 64 + kt * 16 + 2 * t);
				p0[0] = a[kt][0]; p1[0] = a[kt][1]; p0[4] = a[kt][2]; p1[4] = a[kt][3];
			}
		}
		/* output layer: one n-tile (outputs 0..7, 3 used) */
		float o[4];
		o[0] = sb[256 + 2 * t]; o[1] = sb[256 + 2 * t + 1]; o[2] = o[0]; o[3] = o[1];
		#pragma unroll
		for(int kt = 0; kt < 4; kt++) {
			uint32_t w0, w1;
			load_b(W5, LDH, 0, kt * 16, lane, w0, w1);
			mma16816(o, a[kt], w0, w1);
		}
		/* lane (g, t) holds outputs 2t, 2t+1 of rows g and g + 8 */
		#pragma unroll
		for(int half = 0; half < 2; half++) {
			int r = half ? r1 : r0;
			#pragma unroll
			for(int c = 0; c < 2; c++) {
				int col = 2 * t + c;
				float yv = o[2 * half + c];
				if(MODE == FWD_QUERY) {
					if(r < n && col < NRC_O) {
						float4 wv = qo.w[r];
						float wc = col == 0 ? wv.x : (col == 1 ? wv.y : wv.z);
						atomicAdd(reinterpret_cast<float *>(qo.acc + __float_as_int(wv.w)) + col, wc * fmaxf(yv, 0.0f));
					}
				} else if(!TRAIN) {
					if(r < n && col < NRC_O) y[(size_t)r * 3 + col] = yv;
				} else {
					float dy = 0.0f;
					if(r < n && col < NRC_O) {
						float tv = tgt[(size_t)r * 3 + col];
						float den = yv * yv + 0.01f;
						float e = yv - tv;
						loss += e * e / den;
						dy = 2.0f * e / den / (float)(3 * n);
					}
					/* dz5 row r, columns 0..15 (BF16); db5 from the FP32 value */
					tb.dz[5][(size_t)r * 16 + col] = __float2bfloat16_rn(dy);
					db5[c] += dy;
					if(y && r < n && col < NRC_O) y[(size_t)r * 3 + col] = yv;
				}
			}
		}
		if(TRAIN && t < 4) {
			/* columns 8..15 of dz5 are zero padding for the backward MMA k-tile */
			tb.dz[5][(size_t)r0 * 16 + 8 + 2 * t] = __float2bfloat16_rn(0.0f);
			tb.dz[5][(size_t)r0 * 16 + 9 + 2 * t] = __float2bfloat16_rn(0.0f);
			tb.dz[5][(size_t)r1 * 16 + 8 + 2 * t] = __float2bfloat16_rn(0.0f);
			tb.dz[5][(size_t)r1 * 16 + 9 + 2 * t] = __float2bfloat16_rn(0.0f);
		}
	}
	if(TRAIN) {
		for(int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
		if(lane == 0 && loss != 0.0f) atomicAdd(tb.loss, loss / (float)(3 * n));
		/* output-bias gradient: lanes with the same t hold the same columns */
		for(int o = 4; o < 32; o <<= 1) {
			db5[0] += __shfl_xor_sync(0xffffffffu, db5[0], o);
			db5[1] += __shfl_xor_sync(0xffffffffu, db5[1], o);
		}
		if(g == 0) {
			if(2 * t < NRC_O && db5[0] != 0.0f) atomicAdd(&tb.grad[OFF_B5 + 2 * t], db5[0]);
			if(2 * t + 1 < NRC_O && db5[1] != 0.0f) atomicAdd(&tb.grad[OFF_B5 + 2 * t + 1], db5[1]);
		}
	}
}

/* ---- The inference and query forward on the 5th-generation tensor cores ----
 * tcgen05.mma with the accumulators in tensor memory (TMEM).  A CTA of 768
 * threads is three groups of eight warps; each group carries a tile of 128
 * samples through the five layers, two threads per sample (row): its threads
 * write the tile's encoded inputs (half of a row's features each) into
 * shared memory, one elected thread issues the layer's MMAs (M = 128, N = 64,
 * K = 16 each; 14 for the 224-wide first layer, 5 for the 80-wide others,
 * N = 16 for the output layer) and commits them to the group's mbarrier, and
 * the threads read their rows of the accumulator back from TMEM (tcgen05.ld,
 * 32x32b: warp w its lanes 32 (w mod 4) on; the two warps of a lane quarter
 * take 32 columns each) for the ReLU and BF16 rounding that make the next
 * layer's operand, which stays in TMEM (tcgen05.st; the MMA's A operand
 * there, two BF16 per column); the biases come with the products (a BF16 pair
 * per row of each weight tile against a constant pair in the operand).  The
 * features are read only by the first layer, so a group encodes its next
 * tile while the MMAs of the current one's layers 2-5 run (a quarter of the
 * encoding after each of their issues), and the three groups interleave.
 *
 * Shared memory, canonical K-major layouts without swizzle (8-row x 16-byte
 * core matrices; a descriptor's leading byte offset steps along K, its
 * stride byte offset along the rows):
 *   weights   W1 64 x 224, W2-W4 64 x 80, W5 its first 8 rows x 80 (rows 3-7
 *             zero; the MMA's rows 8-15 read the bytes that follow and land in
 *             output columns that are never read), row-group-major: the core
 *             matrices of a row group 128 bytes apart, row groups K/8 x 128
 *   per group the tile's 27 feature chunks, chunk-major: chunk c, row r at
 *             c x 2048 + r x 16 (leading byte offset 2048, stride 128)
 *   constant  2 KB of rows (1, 1, 0 ...), the features' bias pair (chunk 27),
 *             reached by the first layer's last K step through its leading
 *             byte offset
 * 228,648 bytes.  TMEM: 128 columns per group (the hidden accumulator, the
 * hidden operand, the output accumulator).  Every wait on an mbarrier is
 * bounded; one that runs out sets the error word and the group stops at its
 * next barrier (TMEM is released as usual). */
#define TC_NG 3                 /* groups (tiles in flight) per CTA */
#define TC_GROUP_THREADS 256
#define TC_THREADS (TC_NG * TC_GROUP_THREADS)
#define TC_WAIT_LIMIT (1 << 20)
#define TC_XH 5                 /* inputs a half of the encoding reads: 0-4 or 4-8 */

enum {
	TC_KH = 80,                         /* K of layers 2-5: 64 activations, the bias pair, zeros */
	TC_CHUNK = 128 * 16,                /* one 8-element K chunk of a 128-row operand */
	TC_W1 = 0,                          /* 64 x 224: 8 row groups x 28 K-chunks x 128 B */
	TC_W2 = TC_W1 + 64 * NRC_FP * 2,    /* 64 x 80 each */
	TC_W3 = TC_W2 + 64 * TC_KH * 2,
	TC_W4 = TC_W3 + 64 * TC_KH * 2,
	TC_W5 = TC_W4 + 64 * TC_KH * 2,     /* 8 x 80 */
	TC_GROUP0 = TC_W5 + 8 * TC_KH * 2,
	TC_GROUP_BYTES = (NRC_F / 8) * TC_CHUNK,        /* the 27 feature chunks */
	TC_CONST = TC_GROUP0 + TC_NG * TC_GROUP_BYTES,
	TC_MBAR = TC_CONST + TC_CHUNK,
	TC_TMEM_SLOT = TC_MBAR + 8 * TC_NG,
	TC_SMEM = TC_TMEM_SLOT + 16,
	TC_TMEM_COLS = 512,                 /* a power of two >= 128 per group */
	/* a group's TMEM columns, from 128 g: the hidden layers' accumulator,
	 * the hidden operand (80 BF16 = 40 columns), the output layer's
	 * accumulator */
	TC_TD = 0, TC_TA = 64, TC_TO = 112
};
static_assert(TC_SMEM <= 232448, "shared memory of the tensor-core forward");
static_assert(TC_GROUP0 % 128 == 0 && TC_CONST % 128 == 0 && TC_MBAR % 8 == 0, "operand alignment");

/* shared-memory matrix descriptor: start, leading and stride byte offsets, the
 * descriptor version of sm_100, no swizzle */
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
	uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
	d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
	d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
	d |= (uint64_t)1 << 46;
	return d;
}

/* instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, M x N */
__device__ __forceinline__ uint32_t tc_idesc(int m, int n)
{
	return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, int accumulate)
{
	asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
			"tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
			:: "r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate) : "memory");
}

/* the same with the A operand in TMEM (M = 128 lanes, two BF16 per column) */
__device__ __forceinline__ void tc_mma_ta(uint32_t tmem_d, uint32_t tmem_a, uint64_t bdesc, uint32_t idesc, int accumulate)
{
	asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
			"tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}\n"
			:: "r"(tmem_d), "r"(tmem_a), "l"(bdesc), "r"(idesc), "r"(accumulate) : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t mbar)
{
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(mbar) : "memory");
}

__device__ __forceinline__ bool tc_wait(uint32_t mbar, uint32_t parity)
{
	for(int i = 0; i < TC_WAIT_LIMIT; i++) {
		uint32_t done;
		asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.b32 %0, 1, 0, p;\n\t}\n"
				: "=r"(done) : "r"(mbar), "r"(parity) : "memory");
		if(done) return true;
	}
	return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void proxy_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

/* true when v holds in every thread of group g (its named barrier): a wait
 * that ran out in one thread stops the whole group together */
__device__ __forceinline__ bool group_all(int g, bool v)
{
	uint32_t r;
	asm volatile("{\n\t.reg .pred q, p;\n\tsetp.ne.u32 q, %1, 0;\n\tbar.red.and.pred p, %2, %3, q;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
			: "=r"(r) : "r"((uint32_t)v), "r"(1 + g), "n"(TC_GROUP_THREADS) : "memory");
	return r != 0;
}

/* 32 columns of the calling thread's accumulator row (its warp's 32 lanes) */
__device__ __forceinline__ void tc_ld32(uint32_t taddr, float (&v)[32])
{
	uint32_t r[32];
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
			"{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
			: "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
			  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
			  "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
			  "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
			: "r"(taddr) : "memory");
	asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
	#pragma unroll
	for(int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16])
{
	uint32_t r[16];
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
			: "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
			  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
			: "r"(taddr) : "memory");
	asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
	#pragma unroll
	for(int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

/* 16 columns of the calling thread's TMEM lane (its warp's 32 lanes), then
 * the wait for them */
__device__ __forceinline__ void tc_st16(uint32_t taddr, const uint32_t (&r)[16])
{
	asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};"
			:: "r"(taddr), "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
			   "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]) : "memory");
	asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

/* (sin, cos) of a + q quarter turns from (sin a, cos a); q mod 4 in the low bits of q */
__device__ __forceinline__ void quarter_turns(float &s, float &c, uint32_t q)
{
	float s1 = (q & 1u) ? c : s, c1 = (q & 1u) ? s : c;
	s = __uint_as_float(__float_as_uint(s1) ^ ((q << 30) & 0x80000000u));
	c = __uint_as_float(__float_as_uint(c1) ^ (((q + 1u) << 30) & 0x80000000u));
}

/* sin(pi t) and cos(pi t) of two arguments at once in packed FP32 (the
 * .f32x2 operations of sm_100 on), for |t| < 2^20.  Reduction: n = rint(2t)
 * by adding 1.5 x 2^23 (which rounds to an integer and leaves n in the low
 * bits of the sum), r = t - n/2 in [-1/4, 1/4] exactly (one FMA); then
 * sin(pi r) = r P(r^2) and cos(pi r) = 1 + r^2 Q(r^2) with P, Q of degree 3,
 * their coefficients fitted for this kernel by weighted least squares on 4000
 * Chebyshev nodes of [0, 1/4] (relative error of the sine, absolute of the
 * cosine), and n quarter turns.  Error within 8e-8 (against float64 sin and
 * cos of pi t over |t| <= 300, six million points). */
__device__ __forceinline__ void sincospi2(float2 t, float2 &sn, float2 &cs)
{
	const float MAGIC = 12582912.0f;
	const float2 u = __fadd2_rn(__fadd2_rn(t, t), make_float2(MAGIC, MAGIC));
	const float2 n = __fadd2_rn(u, make_float2(-MAGIC, -MAGIC));
	const float2 r = __ffma2_rn(n, make_float2(-0.5f, -0.5f), t);
	const float2 z = __fmul2_rn(r, r);
	float2 p = __ffma2_rn(z, make_float2(-0.5890136361122131f, -0.5890136361122131f),
			make_float2(2.5497612953186035f, 2.5497612953186035f));
	p = __ffma2_rn(p, z, make_float2(-5.167707920074463f, -5.167707920074463f));
	p = __ffma2_rn(p, z, make_float2(3.1415927410125732f, 3.1415927410125732f));
	float2 q = __ffma2_rn(z, make_float2(0.2314295470714569f, 0.2314295470714569f),
			make_float2(-1.3350584506988525f, -1.3350584506988525f));
	q = __ffma2_rn(q, z, make_float2(4.0587077140808105f, 4.0587077140808105f));
	q = __ffma2_rn(q, z, make_float2(-4.934802055358887f, -4.934802055358887f));
	sn = __fmul2_rn(p, r);
	cs = __ffma2_rn(q, z, make_float2(1.0f, 1.0f));
	quarter_turns(sn.x, cs.x, __float_as_uint(u.x));
	quarter_turns(sn.y, cs.y, __float_as_uint(u.y));
}

/* Pairs P0 .. P1 - 1 of this thread's half of a sample's encoded inputs:
 * the half is chunks C0 .. C0 + 13 of the 27 (chunk c = 3v + k holds the
 * (sin, cos) pairs of bands 4k .. 4k + 3 of input v; the bias pair, chunk
 * 27, is the constant block), from inputs C0/3 .. C0/3 + 4 (xv), two chunks
 * (a pair) at a time in packed FP32.  Band 4k from sincospi2 (exact
 * argument scaling), the next three by angle doubling, sin 2a = 2 sin a cos
 * a and cos 2a = 1 - 2 sin^2 a: 0.011 % of the features then round to
 * another BF16 value than the exact ones' (0.009 % from correctly rounded
 * bases). */
template <int C0, int P0, int P1>
__device__ __forceinline__ void tc_encode_pairs(unsigned char *A1, int row, const float (&xv)[TC_XH])
{
	const int v0 = C0 / 3;      /* the first input of this half: 0 or 4 */
	#pragma unroll
	for(int p = P0; p < P1; p++) {
		const int ca = C0 + 2 * p, cb = ca + 1 < NRC_F / 8 ? ca + 1 : ca;
		float2 sn, cs;
		sincospi2(__fmul2_rn(make_float2(xv[ca / 3 - v0], xv[cb / 3 - v0]),
				make_float2((float)(1 << (4 * (ca % 3))), (float)(1 << (4 * (cb % 3))))), sn, cs);
		uint32_t qa[4], qb[4];
		#pragma unroll
		for(int b = 0; b < 4; b++) {
			qa[b] = pack_bf16(sn.x, cs.x);
			qb[b] = pack_bf16(sn.y, cs.y);
			if(b < 3) {
				const float2 m = __fmul2_rn(sn, make_float2(-2.0f, -2.0f));
				const float2 s2 = __fmul2_rn(__fadd2_rn(sn, sn), cs);
				cs = __ffma2_rn(m, sn, make_float2(1.0f, 1.0f));
				sn = s2;
			}
		}
		*reinterpret_cast<uint4 *>(A1 + ca * TC_CHUNK + row * 16) = make_uint4(qa[0], qa[1], qa[2], qa[3]);
		if(cb != ca) *reinterpret_cast<uint4 *>(A1 + cb * TC_CHUNK + row * 16) = make_uint4(qb[0], qb[1], qb[2], qb[3]);
	}
}

template <int P0, int P1>
__device__ __forceinline__ void tc_encode_part(int hf, unsigned char *A1, int row, const float (&xv)[TC_XH])
{
	if(hf) tc_encode_pairs<NRC_FP / 16, P0, P1>(A1, row, xv);
	else tc_encode_pairs<0, P0, P1>(A1, row, xv);
}

/* the inputs of half hf of row `row` (zeros past n) */
__device__ __forceinline__ void tc_inputs(float (&xv)[TC_XH], const float *x, int n, int row, int hf)
{
	#pragma unroll
	for(int k = 0; k < TC_XH; k++) xv[k] = row < n ? x[(size_t)row * 9 + 4 * hf + k] : 0.0f;
}

/* byte offset of element row r, 8-element K-chunk c in the row-group-major layout of a tile with kc chunks */
__device__ __forceinline__ uint32_t tc_canon(int r, int c, int kc) { return (uint32_t)(((r >> 3) * kc + c) * 128 + (r & 7) * 16); }

/* a weight image [rows][ld] (BF16) into the row-group-major layout of kc
 * K-chunks: its first ks chunks, then in chunk ks the row's bias as a BF16
 * pair (hi, lo: b = hi + lo to 2^-17) that multiplies the operand's constant
 * pair (1, 1), the rest zero; rows beyond `rows` up to `rows_pad` zero */
__device__ __forceinline__ void tc_weights(unsigned char *dst, const __nv_bfloat16 *src, int rows, int rows_pad, int ld, int ks, int kc,
		const float *bias)
{
	for(int i = threadIdx.x; i < rows_pad * kc; i += blockDim.x) {
		int r = i / kc, c = i - r * kc;
		uint4 v = make_uint4(0u, 0u, 0u, 0u);
		if(r < rows && c < ks) v = *reinterpret_cast<const uint4 *>(src + (size_t)r * ld + c * 8);
		if(r < rows && c == ks) {
			float b = bias[r];
			__nv_bfloat16 hi = __float2bfloat16_rn(b);
			v.x = pack_bf16(__bfloat162float(hi), b - __bfloat162float(hi));
		}
		*reinterpret_cast<uint4 *>(dst + tc_canon(r, c, kc)) = v;
	}
}

/* two accumulator values as a BF16 pair after ReLU (lo in the low half) */
__device__ __forceinline__ uint32_t relu_bf16x2(float lo, float hi)
{
	uint32_t d;
	asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
	return d;
}

/* half `hf` (32 columns) of the hidden activations of the calling thread's
 * row (the bias came with the product): ReLU and BF16, into columns 16 hf ..
 * 16 hf + 15 of the next layer's operand in TMEM (ta: the operand's first
 * column in the thread's lane quarter) */
__device__ __forceinline__ void tc_hidden(uint32_t ta, int hf, const float (&v)[32])
{
	uint32_t q[16];
	#pragma unroll
	for(int i = 0; i < 16; i++) q[i] = relu_bf16x2(v[2 * i], v[2 * i + 1]);
	tc_st16(ta + (uint32_t)(hf * 16), q);
}

template <int MODE>
__global__ void __launch_bounds__(TC_THREADS, 1) k_nrc_forward_tc(NrcDev net, int n, const float *x, float *y, QueryOut qo,
		unsigned *err)
{
	if(MODE == FWD_QUERY) {
		int c = *qo.count;
		n = c < n ? c : n;
	}
	extern __shared__ __align__(1024) unsigned char tsm[];
	const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(tsm);
	tc_weights(tsm + TC_W1, net.w1, 64, 64, LD1, NRC_F / 8, NRC_FP / 8, net.bias);
	tc_weights(tsm + TC_W2, net.w2, 64, 64, LDH, 8, TC_KH / 8, net.bias + 64);
	tc_weights(tsm + TC_W3, net.w3, 64, 64, LDH, 8, TC_KH / 8, net.bias + 128);
	tc_weights(tsm + TC_W4, net.w4, 64, 64, LDH, 8, TC_KH / 8, net.bias + 192);
	tc_weights(tsm + TC_W5, net.w5, NRC_O, 8, LDH, 8, TC_KH / 8, net.bias + 256);
	for(int i = threadIdx.x; i < TC_CHUNK / 16; i += blockDim.x)
		*reinterpret_cast<uint4 *>(tsm + TC_CONST + i * 16) = make_uint4(pack_bf16(1.0f, 1.0f), 0u, 0u, 0u);
	/* group g: warps 8g .. 8g + 7; a warp's lane quarter (warp mod 4) gives
	 * its rows, its half (hf) the features and accumulator columns it takes */
	const int warp = threadIdx.x >> 5, g = warp >> 3, hf = (warp >> 2) & 1;
	const int tid = ((warp & 3) << 5) | (threadIdx.x & 31);
	const bool leader = (threadIdx.x & (TC_GROUP_THREADS - 1)) == 0;
	unsigned char *A1 = tsm + TC_GROUP0 + g * TC_GROUP_BYTES;
	const uint32_t sA1 = sbase + TC_GROUP0 + g * TC_GROUP_BYTES;
	const uint32_t mbar = sbase + TC_MBAR + 8 * g;
	if(leader) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(mbar) : "memory");
	if(warp == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
				:: "r"(sbase + TC_TMEM_SLOT), "r"((uint32_t)TC_TMEM_COLS) : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
	}
	/* the weights and constants are read by the tensor cores (async proxy) */
	proxy_fence();
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tmem = *reinterpret_cast<const uint32_t *>(tsm + TC_TMEM_SLOT);
	const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;
	const uint32_t tD = tmem + (uint32_t)(g * 128) + TC_TD, tA = tmem + (uint32_t)(g * 128) + TC_TA, tO = tmem + (uint32_t)(g * 128) + TC_TO;
	const uint32_t sW1 = sbase + TC_W1, sW5 = sbase + TC_W5, sK = sbase + TC_CONST;
	const uint32_t id64 = tc_idesc(128, 64), id16 = tc_idesc(128, 16);
	if(hf == 0) {
		/* the hidden operand's last K step: the bias pair (1, 1), then zeros */
		uint32_t q[16] = {pack_bf16(1.0f, 1.0f)};
		tc_st16(tA + lane_off + 32, q);
	}
	uint32_t phase = 0;
	bool ok = true;        /* this thread's waits so far */
	bool agreed = true;    /* the group's, at its last barrier */
	const int ntiles = (n + 127) >> 7, stride = gridDim.x * TC_NG;
	/* The encoding of a group's next tile runs under the MMAs of the
	 * current tile's layers 2-5 (which read the hidden operand, not the
	 * features): a quarter of it after each of their issues.  xv holds the
	 * inputs of the tile to encode next. */
	int tile = blockIdx.x * TC_NG + g;
	float xv[TC_XH];
	tc_inputs(xv, x, n, tile * 128 + tid, hf);
	if(tile < ntiles) tc_encode_part<0, 7>(hf, A1, tid, xv);
	for(; tile < ntiles; tile += stride) {
		const int row = tile * 128 + tid;
		const bool more = tile + stride < ntiles;
		tc_inputs(xv, x, n, row + stride * 128, hf);
		#pragma unroll
		for(int l = 0; l < 5; l++) {
			proxy_fence();
			tc_fence_before();
			agreed = group_all(g, ok);
			if(!agreed) break;
			if(leader) {
				tc_fence_after();
				if(l == 0) {
					for(int j = 0; j < NRC_FP / 16 - 1; j++)
						tc_mma(tD, tc_desc(sA1 + 2 * j * TC_CHUNK, TC_CHUNK, 128), tc_desc(sW1 + j * 256, 128, (NRC_FP / 8) * 128), id64, j);
					/* the last K step: chunk 26, then the constant block's bias pairs */
					const uint32_t a = sA1 + (NRC_F / 8 - 1) * TC_CHUNK;
					tc_mma(tD, tc_desc(a, sK - a, 128), tc_desc(sW1 + (NRC_FP / 16 - 1) * 256, 128, (NRC_FP / 8) * 128), id64, 1);
				} else {
					const uint32_t sW = l < 4 ? sbase + TC_W2 + (uint32_t)(l - 1) * (TC_W3 - TC_W2) : sW5;   /* W2, W3, W4 back to back */
					const uint32_t td = l < 4 ? tD : tO, id = l < 4 ? id64 : id16;
					for(int j = 0; j < TC_KH / 16; j++)
						tc_mma_ta(td, tA + (uint32_t)(8 * j), tc_desc(sW + j * 256, 128, TC_KH / 8 * 128), id, j);
				}
				tc_commit(mbar);
			}
			if(more) {
				if(l == 1) tc_encode_part<0, 2>(hf, A1, tid, xv);
				else if(l == 2) tc_encode_part<2, 4>(hf, A1, tid, xv);
				else if(l == 3) tc_encode_part<4, 6>(hf, A1, tid, xv);
				else if(l == 4) tc_encode_part<6, 7>(hf, A1, tid, xv);
			}
			if(!tc_wait(mbar, phase)) {
				ok = false;     /* phase stays the one still outstanding */
				continue;
			}
			phase ^= 1u;
			tc_fence_after();
			if(l < 4) {
				float v[32];
				tc_ld32(tD + lane_off + (uint32_t)(hf * 32), v);
				tc_hidden(tA + lane_off, hf, v);
			} else if(hf == 0) {
				float v[16];
				tc_ld16(tO + lane_off, v);
				if(row < n) {
					const float *o = v;   /* the bias came with the product */
					if(MODE == FWD_QUERY) {
						float4 wv = qo.w[row];
						float *a = reinterpret_cast<float *>(qo.acc + __float_as_int(wv.w));
						atomicAdd(a, wv.x * fmaxf(o[0], 0.0f));
						atomicAdd(a + 1, wv.y * fmaxf(o[1], 0.0f));
						atomicAdd(a + 2, wv.z * fmaxf(o[2], 0.0f));
					} else {
						y[(size_t)row * 3] = o[0];
						y[(size_t)row * 3 + 1] = o[1];
						y[(size_t)row * 3 + 2] = o[2];
					}
				}
			}
		}
		if(!agreed) break;
	}
	/* the waits of the group's last layer */
	if(agreed) agreed = group_all(g, ok);
	if(!agreed) {
		if(leader) atomicOr(err, 1u);
		/* what was committed may still be running: a last bounded wait by
		 * the threads whose wait ran out (they hold its phase) */
		if(!ok) tc_wait(mbar, phase);
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	if(warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"((uint32_t)TC_TMEM_COLS) : "memory");
}

/* Backward pass, a warp per 16 samples: dH_{l-1} = dZ_l W_l, dZ_{l-1} =
 * dH_{l-1} where h_{l-1} > 0; stores dz[4..1] (BF16) and adds the bias
 * gradients (from the FP32 values) to the packed gradient. */
__global__ void __launch_bounds__(128) k_nrc_backward(NrcDev net, int n, TrainBufs tb)
{
	extern __shared__ __align__(16) unsigned char smem_raw[];
	__nv_bfloat16 *sw = reinterpret_cast<__nv_bfloat16 *>(smem_raw);
	float *sdb = reinterpret_cast<float *>(sw + BWD_SMEM_BF16);   /* 4 x 64 bias sums of the block */
	copy_to_shared(sw, net.w2t, BWD_SMEM_BF16);
	for(int i = threadIdx.x; i < 256; i += blockDim.x) sdb[i] = 0.0f;
	__syncthreads();
	const __nv_bfloat16 *W2T = sw, *W3T = sw + (IMG_W3T - IMG_W2T), *W4T = sw + (IMG_W4T - IMG_W2T), *W5T = sw + (IMG_W5T - IMG_W2T);
	int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	int g = lane >> 2, t = lane & 3;
	int ntiles = (n + 15) >> 4;
	for(int tile = blockIdx.x * 4 + warp; tile < ntiles; tile += gridDim.x * 4) {
		int r0 = tile * 16 + g, r1 = r0 + 8;
		/* dz5 as an A tile (k = outputs, 16 wide) */
		uint32_t a5[4];
		const __nv_bfloat16 *d5 = tb.dz[5];
		a5[0] = *reinterpret_cast<const uint32_t *>(d5 + (size_t)r0 * 16 + 2 * t);
		a5[1] = *reinterpret_cast<const uint32_t *>(d5 + (size_t)r1 * 16 + 2 * t);
		a5[2] = *reinterpret_cast<const uint32_t *>(d5 + (size_t)r0 * 16 + 8 + 2 * t);
		a5[3] = *reinterpret_cast<const uint32_t *>(d5 + (size_t)r1 * 16 + 8 + 2 * t);
		Acc64 dz;
		#pragma unroll
		for(int nt = 0; nt < 8; nt++) {
			dz.d[nt][0] = dz.d[nt][1] = dz.d[nt][2] = dz.d[nt][3] = 0.0f;
			uint32_t w0, w1;
			load_b(W5T, LD5T, nt * 8, 0, lane, w0, w1);
			mma16816(dz.d[nt], a5, w0, w1);
		}
		const __nv_bfloat16 *WT[3] = {W4T, W3T, W2T};
		for(int l = 4; l >= 1; l--) {
			/* mask by h_l > 0, bias sums, BF16 store of dz_l */
			const __nv_bfloat16 *h = tb.h[l];
			__nv_bfloat16 *dzo = tb.dz[l];
			#pragma unroll
			for(int nt = 0; nt < 8; nt++) {
				int col = nt * 8 + 2 * t;
				uint32_t hv0 = *reinterpret_cast<const uint32_t *>(h + (size_t)r0 * 64 + col);
				uint32_t hv1 = *reinterpret_cast<const uint32_t *>(h + (size_t)r1 * 64 + col);
				if(!(bf16_lo(hv0) > 0.0f)) dz.d[nt][0] = 0.0f;
				if(!(bf16_hi(hv0) > 0.0f)) dz.d[nt][1] = 0.0f;
				if(!(bf16_lo(hv1) > 0.0f)) dz.d[nt][2] = 0.0f;
				if(!(bf16_hi(hv1) > 0.0f)) dz.d[nt][3] = 0.0f;
				*reinterpret_cast<uint32_t *>(dzo + (size_t)r0 * 64 + col) = pack_bf16(dz.d[nt][0], dz.d[nt][1]);
				*reinterpret_cast<uint32_t *>(dzo + (size_t)r1 * 64 + col) = pack_bf16(dz.d[nt][2], dz.d[nt][3]);
				float s0 = dz.d[nt][0] + dz.d[nt][2], s1 = dz.d[nt][1] + dz.d[nt][3];
				for(int o = 4; o < 32; o <<= 1) {
					s0 += __shfl_xor_sync(0xffffffffu, s0, o);
					s1 += __shfl_xor_sync(0xffffffffu, s1, o);
				}
				if(g == 0) {
					atomicAdd(&sdb[(l - 1) * 64 + col], s0);
					atomicAdd(&sdb[(l - 1) * 64 + col + 1], s1);
				}
			}
			if(l == 1) break;
			uint32_t a[4][4];
			acc_to_a(dz, a, false);
			const __nv_bfloat16 *W = WT[4 - l];
			#pragma unroll
			for(int nt = 0; nt < 8; nt++) {
				dz.d[nt][0] = dz.d[nt][1] = dz.d[nt][2] = dz.d[nt][3] = 0.0f;
				#pragma unroll
				for(int kt = 0; kt < 4; kt++) {
					uint32_t w0, w1;
					load_b(W, LDH, nt * 8, kt * 16, lane, w0, w1);
					mma16816(dz.d[nt], a[kt], w0, w1);
				}
			}
		}
	}
	__syncthreads();
	const int boff[4] = {OFF_B1, OFF_B2, OFF_B3, OFF_B4};
	for(int i = threadIdx.x; i < 256; i += blockDim.x) {
		float v = sdb[i];
		if(v != 0.0f) atomicAdd(&tb.grad[boff[i >> 6] + (i & 63)], v);
	}
}

/* Weight gradient of one layer over the batch: dW[o][i] = sum_s dz[s][o] h[s][i],
 * M outputs (rows of dz, 16-wide storage stride DZS), N inputs (h stride HS).
 * Samples are split over blocks; each block stages 32 samples at a time,
 * transposed, in shared memory and its 8 warps hold TPW 16x8 output tiles
 * each; the block's sums are added to the packed gradient at OFF (only
 * o < MO, i < NI are real). */
template <int MT, int NT, int TPW, int DZS, int HS>
__global__ void __launch_bounds__(256) k_nrc_wgrad(int n, const __nv_bfloat16 *dz, const __nv_bfloat16 *h, float *grad, int off,
		int MO, int NI, int per_block)
{
	enum { M = MT * 16, N = NT * 8, LDS = 40 };
	__shared__ __align__(16) __nv_bfloat16 sdz[M * LDS];
	__shared__ __align__(16) __nv_bfloat16 sh[N * LDS];
	int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	int g = lane >> 2, t = lane & 3;
	float acc[TPW][4];
	#pragma unroll
	for(int k = 0; k < TPW; k++) acc[k][0] = acc[k][1] = acc[k][2] = acc[k][3] = 0.0f;
	int s_begin = blockIdx.x * per_block, s_end = min(n, s_begin + per_block);
	for(int s0 = s_begin; s0 < s_end; s0 += 32) {
		__syncthreads();
		/* stage dz^T [M][32] and h^T [N][32] */
		for(int i = threadIdx.x; i < 32 * M; i += blockDim.x) {
			int s = i / M, o = i - s * M;
			__nv_bfloat16 v = __float2bfloat16_rn(0.0f);
			if(s0 + s < s_end && o < DZS) v = dz[(size_t)(s0 + s) * DZS + o];
			sdz[o * LDS + s] = v;
		}
		for(int i = threadIdx.x; i < 32 * N; i += blockDim.x) {
			int s = i / N, c = i - s * N;
			__nv_bfloat16 v = __float2bfloat16_rn(0.0f);
			if(s0 + s < s_end && c < HS) v = h[(size_t)(s0 + s) * HS + c];
			sh[c * LDS + s] = v;
		}
		__syncthreads();
		#pragma unroll
		for(int k = 0; k < TPW; k++) {
			int tile = warp * TPW + k;
			if(tile >= MT * NT) break;
			int mt = tile / NT, nt = tile - mt * NT;
			#pragma unroll
			for(int ks = 0; ks < 2; ks++) {
				uint32_t a[4];
				const __nv_bfloat16 *pa = sdz + (mt * 16 + g) * LDS + ks * 16 + 2 * t;
				a[0] = *reinterpret_cast<const uint32_t *>(pa);
				a[1] = *reinterpret_cast<const uint32_t *>(pa + 8 * LDS);
				a[2] = *reinterpret_cast<const uint32_t *>(pa + 8);
				a[3] = *reinterpret_cast<const uint32_t *>(pa + 8 * LDS + 8);
				uint32_t b0, b1;
				load_b(sh, LDS, nt * 8, ks * 16, lane, b0, b1);
				mma16816(acc[k], a, b0, b1);
			}
		}
	}
	#pragma unroll
	for(int k = 0; k < TPW; k++) {
		int tile = warp * TPW + k;
		if(tile >= MT * NT) break;
		int mt = tile / NT, nt = tile - mt * NT;
		int rows[2] = {mt * 16 + g, mt * 16 + g + 8};
		#pragma unroll
		for(int half = 0; half < 2; half++) {
			int o = rows[half];
			#pragma unroll
			for(int c = 0; c < 2; c++) {
				int i = nt * 8 + 2 * t + c;
				float v = acc[k][2 * half + c];
				if(o < MO && i < NI && v != 0.0f) atomicAdd(&grad[off + o * NI + i], v);
			}
		}
	}
}

/* Adam on the FP32 master; the BF16 images are rewritten from it */
__global__ void k_nrc_adam(float *p, float *m, float *v, float *grad, const int *step_dev, float lr)
{
	const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
	int step = *step_dev + 1;   /* the step counter lives on the device, so that a captured graph replays */
	float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < NRC_NPARAM; i += gridDim.x * blockDim.x) {
		float gi = grad[i];
		grad[i] = 0.0f;
		float mi = b1 * m[i] + (1.0f - b1) * gi;
		float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
		m[i] = mi;
		v[i] = vi;
		float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
		p[i] = pi;
	}
}

/* the BF16 images and FP32 biases of the current master weights; after an
 * Adam step (count_step) also the step counter */
__global__ void k_nrc_images(const float *p, __nv_bfloat16 *img, float *bias, int *step_dev, int count_step)
{
	if(count_step && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(step_dev, 1);
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < IMG_END; i += gridDim.x * blockDim.x) {
		float v = 0.0f;
		if(i < IMG_W2) {
			int o = i / LD1, c = i - o * LD1;
			if(c < NRC_F) v = p[OFF_W1 + o * NRC_F + c];
		} else if(i < IMG_W5) {
			int l = (i - IMG_W2) / (64 * LDH), r = i - IMG_W2 - l * 64 * LDH;
			int o = r / LDH, c = r - o * LDH;
			const int offs[3] = {OFF_W2, OFF_W3, OFF_W4};
			if(c < 64) v = p[offs[l] + o * 64 + c];
		} else if(i < IMG_W2T) {
			int r = i - IMG_W5, o = r / LDH, c = r - o * LDH;
			if(o < NRC_O && c < 64) v = p[OFF_W5 + o * 64 + c];
		} else if(i < IMG_W5T) {
			int l = (i - IMG_W2T) / (64 * LDH), r = i - IMG_W2T - l * 64 * LDH;
			int in = r / LDH, o = r - in * LDH;
			const int offs[3] = {OFF_W2, OFF_W3, OFF_W4};
			if(o < 64) v = p[offs[l] + o * 64 + in];
		} else {
			int r = i - IMG_W5T, in = r / LD5T, o = r - in * LD5T;
			if(o < NRC_O) v = p[OFF_W5 + o * 64 + in];
		}
		img[i] = __float2bfloat16_rn(v);
	}
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < NRC_NBIAS; i += gridDim.x * blockDim.x) {
		float v = 0.0f;
		if(i < 256) {
			const int offs[4] = {OFF_B1, OFF_B2, OFF_B3, OFF_B4};
			v = p[offs[i >> 6] + (i & 63)];
		} else if(i - 256 < NRC_O) {
			v = p[OFF_B5 + i - 256];
		}
		bias[i] = v;
	}
}

/* ---------------- host side ---------------- */

struct NrcState {
	int device = -1;
	float *p = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr, *loss = nullptr, *bias = nullptr;
	int *step_dev = nullptr;         /* Adam steps taken (device copy of `step`) */
	unsigned *tc_err = nullptr;      /* set when a tensor-core forward's bounded wait ran out */
	int nsm = 0;
	/* the per-frame training steps as a CUDA graph, replayed while the
	 * batch shape and buffers stay the same */
	cudaGraphExec_t graph = nullptr;
	cudaStream_t cap = nullptr;      /* stream the graph is captured on (the caller's may be the legacy stream) */
	int g_steps = 0, g_per = 0;
	const float *g_x = nullptr, *g_t = nullptr;
	float g_lr = 0.0f;
	__nv_bfloat16 *img = nullptr;
	__nv_bfloat16 *hbuf = nullptr;   /* training activations */
	int hcap = 0;                    /* samples the training buffers hold */
	int step = 0;
	bool ready = false;
	std::string err;
};

static NrcState g_nrc;
static std::mutex g_nrc_mu;

static int nrc_fail(cudaError_t e, const char *where)
{
	g_nrc.err = std::string(where) + ": " + cudaGetErrorString(e);
	return SRAY_ECUDA;
}

#define NCK(call, where) do { cudaError_t e_ = (call); if(e_ != cudaSuccess) return nrc_fail(e_, where); } while(0)

static NrcDev nrc_dev()
{
	NrcDev d;
	const __nv_bfloat16 *b = g_nrc.img;
	d.w1 = b + IMG_W1; d.w2 = b + IMG_W2; d.w3 = b + IMG_W3; d.w4 = b + IMG_W4; d.w5 = b + IMG_W5;
	d.w2t = b + IMG_W2T; d.w3t = b + IMG_W3T; d.w4t = b + IMG_W4T; d.w5t = b + IMG_W5T;
	d.bias = g_nrc.bias;
	return d;
}

static int nrc_alloc()
{
	int dev = 0;
	NCK(cudaGetDevice(&dev), "device");
	if(g_nrc.ready && g_nrc.device == dev) return 0;
	NCK(cudaMalloc(&g_nrc.p, NRC_NPARAM * sizeof(float)), "radiance cache weights");
	NCK(cudaMalloc(&g_nrc.m, NRC_NPARAM * sizeof(float)), "radiance cache moments");
	NCK(cudaMalloc(&g_nrc.v, NRC_NPARAM * sizeof(float)), "radiance cache moments");
	NCK(cudaMalloc(&g_nrc.grad, NRC_NPARAM * sizeof(float)), "radiance cache gradient");
	NCK(cudaMalloc(&g_nrc.loss, sizeof(float)), "radiance cache loss");
	NCK(cudaMalloc(&g_nrc.bias, NRC_NBIAS * sizeof(float)), "radiance cache biases");
	NCK(cudaMalloc(&g_nrc.img, IMG_END * sizeof(__nv_bfloat16)), "radiance cache images");
	NCK(cudaMalloc(&g_nrc.step_dev, sizeof(int)), "radiance cache step");
	NCK(cudaMalloc(&g_nrc.tc_err, sizeof(unsigned)), "radiance cache error word");
	NCK(cudaMemset(g_nrc.tc_err, 0, sizeof(unsigned)), "radiance cache error word");
	NCK(cudaDeviceGetAttribute(&g_nrc.nsm, cudaDevAttrMultiProcessorCount, dev), "multiprocessors");
	NCK(cudaFuncSetAttribute(k_nrc_forward_tc<FWD_INFER>, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM), "smem");
	NCK(cudaFuncSetAttribute(k_nrc_forward_tc<FWD_QUERY>, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM), "smem");
	NCK(cudaFuncSetAttribute(k_nrc_forward<FWD_TRAIN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
			FWD_SMEM_BF16 * 2 + NRC_NBIAS * 4), "smem");
	NCK(cudaFuncSetAttribute(k_nrc_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, BWD_SMEM_BF16 * 2 + 256 * 4), "smem");
	g_nrc.device = dev;
	g_nrc.ready = true;
	return 0;
}

static int nrc_set(const float *host_p, cudaStream_t s)
{
	NCK(cudaMemcpyAsync(g_nrc.p, host_p, NRC_NPARAM * sizeof(float), cudaMemcpyHostToDevice, s), "upload weights");
	NCK(cudaMemsetAsync(g_nrc.m, 0, NRC_NPARAM * sizeof(float), s), "reset moments");
	NCK(cudaMemsetAsync(g_nrc.v, 0, NRC_NPARAM * sizeof(float), s), "reset moments");
	NCK(cudaMemsetAsync(g_nrc.grad, 0, NRC_NPARAM * sizeof(float), s), "reset gradient");
	NCK(cudaMemsetAsync(g_nrc.step_dev, 0, sizeof(int), s), "reset step");
	k_nrc_images<<<64, 256, 0, s>>>(g_nrc.p, g_nrc.img, g_nrc.bias, g_nrc.step_dev, 0);
	NCK(cudaGetLastError(), "radiance cache images");
	g_nrc.step = 0;
	return 0;
}

/* He-uniform weights from a Philox stream, zero biases */
static void nrc_init_host(uint64_t seed, std::vector<float> &p)
{
	p.assign(NRC_NPARAM, 0.0f);
	struct L { int off, out, in; } ls[5] = {{OFF_W1, 64, NRC_F}, {OFF_W2, 64, 64}, {OFF_W3, 64, 64}, {OFF_W4, 64, 64}, {OFF_W5, 3, 64}};
	sray_rng r;
	sray_rng_init(&r, seed, SRAY_DOM_USER, 0x4e5243u, 0);
	for(const L &l : ls) {
		float lim = sqrtf(6.0f / (float)l.in);
		for(int i = 0; i < l.out * l.in; i++) p[l.off + i] = (2.0f * sray_rng_uniform_f(&r) - 1.0f) * lim;
	}
}

static int nrc_train_bufs(int n, TrainBufs &tb, cudaStream_t s)
{
	int n16 = (n + 15) & ~15;
	if(n16 > g_nrc.hcap) {
		if(g_nrc.hbuf) cudaFree(g_nrc.hbuf);
		g_nrc.hbuf = nullptr;
		g_nrc.hcap = 0;
		size_t per = NRC_FP + 4 * 64 + 4 * 64 + 16;
		NCK(cudaMalloc(&g_nrc.hbuf, (size_t)n16 * per * sizeof(__nv_bfloat16)), "radiance cache training buffers");
		g_nrc.hcap = n16;
	}
	__nv_bfloat16 *b = g_nrc.hbuf;
	size_t cap = (size_t)g_nrc.hcap;
	tb.h[0] = b; b += cap * NRC_FP;
	for(int l = 1; l <= 4; l++) { tb.h[l] = b; b += cap * 64; }
	tb.dz[0] = nullptr;
	for(int l = 1; l <= 4; l++) { tb.dz[l] = b; b += cap * 64; }
	tb.dz[5] = b;
	tb.grad = g_nrc.grad;
	tb.loss = g_nrc.loss;
	(void)s;
	return 0;
}

/* blocks for n samples at wpb warps per block (16 samples per warp); at
 * most a few resident waves, the kernels loop over the rest */
static int nrc_grid(int n, int wpb)
{
	int tiles = (n + 15) / 16;
	int blocks = (tiles + wpb - 1) / wpb;
	int cap = 152 * 32 / wpb;
	if(blocks > cap) blocks = cap;
	return blocks < 1 ? 1 : blocks;
}

/* gradient of the loss over a batch into g_nrc.grad (which must hold zeros) */
static int nrc_gradient(int n, const float *x, const float *t, float *y, cudaStream_t s)
{
	TrainBufs tb;
	int r = nrc_train_bufs(n, tb, s);
	if(r) return r;
	NCK(cudaMemsetAsync(g_nrc.loss, 0, sizeof(float), s), "reset loss");
	NrcDev d = nrc_dev();
	k_nrc_forward<FWD_TRAIN><<<nrc_grid(n, NRC_FWD_THREADS / 32), NRC_FWD_THREADS, FWD_SMEM_BF16 * 2 + NRC_NBIAS * 4, s>>>(d, n, x, y, t,
			tb, QueryOut());
	k_nrc_backward<<<nrc_grid(n, 4), 128, BWD_SMEM_BF16 * 2 + 256 * 4, s>>>(d, n, tb);
	/* samples per weight-gradient block: about two blocks per SM, at least
	 * 128 (each block adds its partial dW with atomics) */
	int per = (n + 2 * 152 - 1) / (2 * 152);
	per = per < 128 ? 128 : (per + 31) & ~31;
	int blocks = (n + per - 1) / per;
	/* layer 1: 64 x 224 (216 real), layers 2-4: 64 x 64, layer 5: 16 x 64 (3 real) */
	k_nrc_wgrad<4, 28, 14, 64, NRC_FP><<<blocks, 256, 0, s>>>(n, tb.dz[1], tb.h[0], g_nrc.grad, OFF_W1, 64, NRC_F, per);
	k_nrc_wgrad<4, 8, 4, 64, 64><<<blocks, 256, 0, s>>>(n, tb.dz[2], tb.h[1], g_nrc.grad, OFF_W2, 64, 64, per);
	k_nrc_wgrad<4, 8, 4, 64, 64><<<blocks, 256, 0, s>>>(n, tb.dz[3], tb.h[2], g_nrc.grad, OFF_W3, 64, 64, per);
	k_nrc_wgrad<4, 8, 4, 64, 64><<<blocks, 256, 0, s>>>(n, tb.dz[4], tb.h[3], g_nrc.grad, OFF_W4, 64, 64, per);
	k_nrc_wgrad<1, 8, 1, 16, 64><<<blocks, 256, 0, s>>>(n, tb.dz[5], tb.h[4], g_nrc.grad, OFF_W5, NRC_O, 64, per);
	NCK(cudaGetLastError(), "radiance cache gradient");
	return 0;
}

int nrc_ensure_ready(uint64_t seed, cudaStream_t s)
{
	bool fresh = !g_nrc.ready;
	int r = nrc_alloc();
	if(r) return r;
	if(fresh) {
		std::vector<float> p;
		nrc_init_host(seed, p);
		if((r = nrc_set(p.data(), s))) return r;
		NCK(cudaStreamSynchronize(s), "radiance cache init");
	}
	return 0;
}

/* CTAs of the tensor-core forward for up to n samples: one per SM at
 * most, TC_NG 128-sample tiles in flight each */
static int tc_grid(int n)
{
	int tiles = (n + 127) / 128;
	int blocks = (tiles + TC_NG - 1) / TC_NG;
	int cap = g_nrc.nsm > 0 ? g_nrc.nsm : 152;
	if(blocks > cap) blocks = cap;
	return blocks < 1 ? 1 : blocks;
}

int nrc_infer(int n, const float *x, float *y, cudaStream_t s)
{
	if(n <= 0) return 0;
	k_nrc_forward_tc<FWD_INFER><<<tc_grid(n), TC_THREADS, TC_SMEM, s>>>(nrc_dev(), n, x, y, QueryOut(), g_nrc.tc_err);
	NCK(cudaGetLastError(), "radiance cache inference");
	return 0;
}

int nrc_device_error(cudaStream_t s)
{
	if(!g_nrc.ready) return 0;
	unsigned h = 0;
	NCK(cudaMemcpyAsync(&h, g_nrc.tc_err, sizeof h, cudaMemcpyDeviceToHost, s), "radiance cache error word");
	NCK(cudaStreamSynchronize(s), "radiance cache error word");
	if(h) {
		g_nrc.err = "radiance cache: a tensor-core wait ran out";
		NCK(cudaMemsetAsync(g_nrc.tc_err, 0, sizeof(unsigned), s), "radiance cache error word");
		return SRAY_EDEVICE;
	}
	return 0;
}

int nrc_query(const int *count, int cap, const float *x, const float4 *w, float4 *acc, cudaStream_t s)
{
	if(cap <= 0) return 0;
	QueryOut qo;
	qo.count = count;
	qo.w = w;
	qo.acc = acc;
	k_nrc_forward_tc<FWD_QUERY><<<tc_grid(cap), TC_THREADS, TC_SMEM, s>>>(nrc_dev(), cap, x, nullptr, qo, g_nrc.tc_err);
	NCK(cudaGetLastError(), "radiance cache queries");
	return 0;
}

int nrc_train(int n, const float *x, const float *t, float lr, cudaStream_t s)
{
	if(n <= 0) return 0;
	int r = nrc_gradient(n, x, t, nullptr, s);
	if(r) return r;
	g_nrc.step++;
	k_nrc_adam<<<64, 256, 0, s>>>(g_nrc.p, g_nrc.m, g_nrc.v, g_nrc.grad, g_nrc.step_dev, lr);
	k_nrc_images<<<64, 256, 0, s>>>(g_nrc.p, g_nrc.img, g_nrc.bias, g_nrc.step_dev, 1);
	NCK(cudaGetLastError(), "radiance cache training");
	return 0;
}

/* `steps` Adam steps over consecutive batches of `per` samples: captured
 * once as a CUDA graph (forward, backward, weight gradients, Adam and weight
 * images of every step: steps * NRC_TRAIN_KERNELS kernels) and replayed
 * while the shape, buffers and rate stay the same */
int nrc_train_steps(int steps, int per, const float *x, const float *t, float lr, cudaStream_t s)
{
	if(steps <= 0 || per <= 0) return 0;
	NrcState &G = g_nrc;
	if(!(G.graph && G.g_steps == steps && G.g_per == per && G.g_x == x && G.g_t == t && G.g_lr == lr)) {
		if(G.graph) {
			cudaGraphExecDestroy(G.graph);
			G.graph = nullptr;
		}
		TrainBufs tb;
		int r = nrc_train_bufs(per, tb, s);   /* allocate before the capture */
		if(r) return r;
		if(!G.cap) NCK(cudaStreamCreateWithFlags(&G.cap, cudaStreamNonBlocking), "capture stream");
		cudaGraph_t g = nullptr;
		NCK(cudaStreamBeginCapture(G.cap, cudaStreamCaptureModeThreadLocal), "capture training steps");
		int step0 = G.step;
		for(int i = 0; i < steps && !r; i++) r = nrc_train(per, x + (size_t)i * per * 9, t + (size_t)i * per * 3, lr, G.cap);
		G.step = step0;
		cudaError_t e = cudaStreamEndCapture(G.cap, &g);
		if(r) {
			if(g) cudaGraphDestroy(g);
			return r;
		}
		if(e != cudaSuccess) return nrc_fail(e, "capture training steps");
		e = cudaGraphInstantiate(&G.graph, g, 0);
		cudaGraphDestroy(g);
		if(e != cudaSuccess) {
			G.graph = nullptr;
			return nrc_fail(e, "instantiate training graph");
		}
		G.g_steps = steps;
		G.g_per = per;
		G.g_x = x;
		G.g_t = t;
		G.g_lr = lr;
	}
	NCK(cudaGraphLaunch(G.graph, s), "training graph");
	G.step += steps;
	return 0;
}

const char *nrc_error() { return g_nrc.err.c_str(); }

float *nrc_loss_ptr() { return g_nrc.loss; }

}  // namespace sray

using namespace sray;

extern "C" {

static thread_local std::string t_nrc_err;

static int nrc_err_ret(int r)
{
	if(r) t_nrc_err = g_nrc.err;
	return r;
}

int sray_nrc_reset(uint64_t seed)
{
	std::lock_guard<std::mutex> lk(g_nrc_mu);
	int r = nrc_alloc();
	if(r) return nrc_err_ret(r);
	std::vector<float> p;
	nrc_init_host(seed, p);
	r = nrc_set(p.data(), 0);
	if(!r) { cudaError_t e = cudaStreamSynchronize(0); if(e != cudaSuccess) r = nrc_fail(e, "reset"); }
	return nrc_err_ret(r);
}

int sray_nrc_set_params(const float *p, int n)
{
	std::lock_guard<std::mutex> lk(g_nrc_mu);
	if(!p || n != NRC_NPARAM) { g_nrc.err = "expected SRAY_NRC_PARAMS parameters"; return nrc_err_ret(SRAY_EINVAL); }
	int r = nrc_alloc();
	if(!r) r = nrc_set(p, 0);
	if(!r) { cudaError_t e = cudaStreamSynchronize(0); if(e != cudaSuccess) r = nrc_fail(e, "set parameters"); }
	return nrc_err_ret(r);
}

int sray_nrc_get_params(float *p, int n)
{
	std::lock_guard<std::mutex> lk(g_nrc_mu);
	if(!p || n != NRC_NPARAM) { g_nrc.err = "expected SRAY_NRC_PARAMS parameters"; return nrc_err_ret(SRAY_EINVAL); }
	if(!g_nrc.ready) { g_nrc.err = "radiance cache not initialised"; return nrc_err_ret(SRAY_ESTATE); }
	cudaError_t e = cudaMemcpy(p, g_nrc.p, NRC_NPARAM * sizeof(float), cudaMemcpyDeviceToHost);
	return nrc_err_ret(e == cudaSuccess ? 0 : nrc_fail(e, "get parameters"));
}

int sray_nrc_infer(int n, const float *x, float *y, void *stream)
{
	std::lock_guard<std::mutex> lk(g_nrc_mu);
	if(n < 0 || (n > 0 && (!x || !y))) { g_nrc.err = "bad arguments"; return nrc_err_ret(SRAY_EINVAL); }
	if(!g_nrc.ready) { g_nrc.err = "radiance cache not initialised"; return nrc_err_ret(SRAY_ESTATE); }
	cudaStream_t s = (cudaStream_t)stream;
	int r = nrc_infer(n, x, y, s);
	if(!r) { cudaError_t e = cudaStreamSynchronize(s); if(e != cudaSuccess) r = nrc_fail(e, "inference"); }
	if(!r) r = nrc_device_error(s);
	return nrc_err_ret(r);
}

int sray_nrc_infer_async(int n, const float *x, float *y, void *stream)
{
	std::lock_guard<std::mutex> lk(g_nrc_mu);
	if(n < 0 || (n > 0 && (!x || !y))) { g_nrc.err = "bad arguments"; return nrc_err_ret(SRAY_EINVAL); }
	if(!g_nrc.ready) { g_nrc.err = "radiance cache not initialised"; return nrc_err_ret(SRAY_ESTATE); }
	return nrc_err_ret(nrc_infer(n, x, y, (cudaStream_t)stream));
}

int sray_nrc_check(void *stream)
{
	std::lock_guard<std::mutex> lk(g_nrc_mu);
	if(!g_nrc.ready) return 0;
	cudaStream_t s = (cudaStream_t)stream;
	int r = 0;
	cudaError_t e = cudaStreamSynchronize(s);
	if(e != cudaSuccess) r = nrc_fail(e, "inference");
	if(!r) r = nrc_device_error(s);
	return nrc_err_ret(r);
}

int sray_nrc_gradients(int n, const float *x, const float *t, float *grad, float *loss, void *stream)
{
	std::lock_guard<std::mutex> lk(g_nrc_mu);
	if(n <= 0 || !x || !t || !grad || !loss) { g_nrc.err = "bad arguments"; return nrc_err_ret(SRAY_EINVAL); }
	if(!g_nrc.ready) { g_nrc.err = "radiance cache not initialised"; return nrc_err_ret(SRAY_ESTATE); }
	cudaStream_t s = (cudaStream_t)stream;
	int r = 0;
	cudaError_t e = cudaMemsetAsync(g_nrc.grad, 0, NRC_NPARAM * sizeof(float), s);
	if(e != cudaSuccess) r = nrc_fail(e, "reset gradient");
	if(!r) r = nrc_gradient(n, x, t, nullptr, s);
	if(!r) { e = cudaMemcpyAsync(grad, g_nrc.grad, NRC_NPARAM * sizeof(float), cudaMemcpyDeviceToDevice, s); if(e != cudaSuccess) r = nrc_fail(e, "copy gradient"); }
	if(!r) { e = cudaMemcpyAsync(loss, g_nrc.loss, sizeof(float), cudaMemcpyDeviceToDevice, s); if(e != cudaSuccess) r = nrc_fail(e, "copy loss"); }
	if(!r) { e = cudaMemsetAsync(g_nrc.grad, 0, NRC_NPARAM * sizeof(float), s); if(e != cudaSuccess) r = nrc_fail(e, "reset gradient"); }
	if(!r) { e = cudaStreamSynchronize(s); if(e != cudaSuccess) r = nrc_fail(e, "gradients"); }
	return nrc_err_ret(r);
}

int sray_nrc_train(int n, const float *x, const float *t, float *loss, void *stream)
{
	std::lock_guard<std::mutex> lk(g_nrc_mu);
	if(n <= 0 || !x || !t) { g_nrc.err = "bad arguments"; return nrc_err_ret(SRAY_EINVAL); }
	if(!g_nrc.ready) { g_nrc.err = "radiance cache not initialised"; return nrc_err_ret(SRAY_ESTATE); }
	cudaStream_t s = (cudaStream_t)stream;
	int r = nrc_train(n, x, t, 1e-3f, s);
	if(!r && loss) { cudaError_t e = cudaMemcpyAsync(loss, g_nrc.loss, sizeof(float), cudaMemcpyDeviceToDevice, s); if(e != cudaSuccess) r = nrc_fail(e, "copy loss"); }
	if(!r) { cudaError_t e = cudaStreamSynchronize(s); if(e != cudaSuccess) r = nrc_fail(e, "training"); }
	return nrc_err_ret(r);
}

int sray_nrc_last_error(char *buf, size_t len)
{
	if(!buf || len == 0) return SRAY_EINVAL;
	size_t n = t_nrc_err.size() < len - 1 ? t_nrc_err.size() : len - 1;
	memcpy(buf, t_nrc_err.data(), n);
	buf[n] = 0;
	return 0;
}

}  /* extern "C" */
