// Pixel-parallel kernels over the fragment store (no reference counterpart).
//
// In store mode the raster pass writes every pixel's fragments, in exact blend order (nearest
// first, ties by primitive id), as tri slots to a fragment store, and skips shading and
// blending. These kernels then work one thread per pixel, many warps per SM, so that the
// per-fragment loads of shading overlap the serial per-pixel blend:
//
//  blendPixelsKernel   the plain forward's blend (shading.glsl:272-285, 312): FP32
//                      out += rgb*a*T; T *= 1-a, stop at T == 0 (or T < 1/128 with the alpha
//                      threshold), additive variant, background, saturate. Same operations in
//                      the same order as the raster pass's own blend, so the same image bits.
//  gradColorKernel     shades the pixel's stored fragments (the raster's shadeFragment, same
//                      FP32 colour) and accumulates the colour in FP64 with an FP64
//                      transmittance, stopping where the FP32 transmittance of the image reaches
//                      0; writes clamp(FP64 colour rounded to FP32) as the image.
//  gradBackwardKernel  replays the same list front to back and routes dL/dimage to the vertex
//                      colours and triangle opacities: dC/dc_i = a_i T_i and
//                      dC/da_i = c_i T_i - S_i / (1 - a_i), S_i = C - (colour accumulated up to and
//                      including fragment i), in FP64.
//
// Both run only when the store held the whole frame (grad_state[0] == 0); otherwise the raster
// pass's FP64 colour and backward modes recompute the fragment lists instead.

#include "lucid_common.cuh"
#include "lucid_kernels.h"
#include "lucid_shade.cuh"

namespace lucid {

constexpr int kGradTileX = 32, kGradTileY = 8;

__device__ __forceinline__ bool gradStoreComplete(const FrameParams& p) {
	return *reinterpret_cast<const volatile unsigned long long*>(p.grad_state) == 0ull;
}

__global__ void __launch_bounds__(kGradTileX * kGradTileY) blendPixelsKernel(FrameParams p) {
	if(!gradStoreComplete(p))
		return;
	const int x = blockIdx.x * kGradTileX + threadIdx.x, y = blockIdx.y * kGradTileY + threadIdx.y;
	if(x >= p.width || y >= p.height)
		return;
	const size_t pix = size_t(y) * p.width + x;
	const uint32_t off = p.grad_px_off[pix], cnt = p.grad_px_cnt[pix];
	const bool additive = (p.flags & LUCID_OPT_ADDITIVE_BLENDING) != 0;
	const bool alpha_threshold = (p.flags & LUCID_OPT_ALPHA_THRESHOLD) != 0;
	float c0 = 0.0f, c1 = 0.0f, c2 = 0.0f, T = 1.0f;
	for(uint32_t j = 0; j < cnt; j++) {
		const uint32_t tri = p.grad_tris[off + j];
		if(tri >= 2u * uint32_t(p.max_visible_quads))
			continue; // only after a device error (the frame's lucid_info has it)
		const float4 c = shadeFragment(p, tri, fragmentDepth(p, tri, x, y), x, y);
		if(additive) {
			c0 = c0 + c.x * c.w;
			c1 = c1 + c.y * c.w;
			c2 = c2 + c.z * c.w;
		} else {
			c0 = c0 + (c.x * c.w) * T;
			c1 = c1 + (c.y * c.w) * T;
			c2 = c2 + (c.z * c.w) * T;
			T = T * (1.0f - c.w);
			if(T == 0.0f || (alpha_threshold && T < (1.0f / 128.0f)))
				break;
		}
	}
	const float* bg = p.cfg.background_color;
	float4 o;
	o.x = fminf(fmaxf(c0 + T * bg[0], 0.0f), 1.0f);
	o.y = fminf(fmaxf(c1 + T * bg[1], 0.0f), 1.0f);
	o.z = fminf(fmaxf(c2 + T * bg[2], 0.0f), 1.0f);
	o.w = 1.0f;
	reinterpret_cast<float4*>(p.out_rgba)[pix] = o;
}

__global__ void __launch_bounds__(kGradTileX * kGradTileY) gradColorKernel(FrameParams p) {
	if(!gradStoreComplete(p))
		return;
	const int x = blockIdx.x * kGradTileX + threadIdx.x, y = blockIdx.y * kGradTileY + threadIdx.y;
	if(x >= p.width || y >= p.height)
		return;
	const size_t pix = size_t(y) * p.width + x;
	const uint32_t off = p.grad_px_off[pix], cnt = p.grad_px_cnt[pix];
	double acc[3] = {0.0, 0.0, 0.0}, T64 = 1.0;
	float T = 1.0f;
	for(uint32_t j = 0; j < cnt; j++) {
		const uint32_t tri = p.grad_tris[off + j];
		if(tri >= 2u * uint32_t(p.max_visible_quads))
			continue; // only after a device error (the frame's lucid_info has it)
		const float4 c = shadeFragment(p, tri, fragmentDepth(p, tri, x, y), x, y);
		acc[0] += double(c.x * c.w) * T64;
		acc[1] += double(c.y * c.w) * T64;
		acc[2] += double(c.z * c.w) * T64;
		T64 *= 1.0 - double(c.w);
		T = T * (1.0f - c.w);
		if(T == 0.0f)
			break;
	}
	float out[3];
	for(int ch = 0; ch < 3; ch++) {
		const double col = acc[ch] + T64 * double(p.cfg.background_color[ch]);
		p.px_color64[pix * 3 + ch] = col;
		const float cf = float(col);
		p.px_color32[pix * 3 + ch] = cf;
		out[ch] = fminf(fmaxf(cf, 0.0f), 1.0f);
	}
	reinterpret_cast<float4*>(p.out_rgba)[pix] = make_float4(out[0], out[1], out[2], 1.0f);
}

__global__ void __launch_bounds__(kGradTileX * kGradTileY) gradBackwardKernel(FrameParams p) {
	if(!gradStoreComplete(p))
		return;
	const int x = blockIdx.x * kGradTileX + threadIdx.x, y = blockIdx.y * kGradTileY + threadIdx.y;
	if(x >= p.width || y >= p.height)
		return;
	const size_t pix = size_t(y) * p.width + x;
	// dL/dC through the clamp of the output (gradient passes where 0 <= C <= 1)
	float grad[3];
	double c64[3];
	bool any = false;
	for(int ch = 0; ch < 3; ch++) {
		const float cf = p.px_color32[pix * 3 + ch];
		const float g = p.dl_dimage[pix * 4 + ch];
		grad[ch] = (cf >= 0.0f && cf <= 1.0f) ? g : 0.0f;
		c64[ch] = p.px_color64[pix * 3 + ch];
		any |= grad[ch] != 0.0f;
	}
	if(!any)
		return;
	const uint32_t off = p.grad_px_off[pix], cnt = p.grad_px_cnt[pix];
	const bool vertex_grads = p.dvertex_rgba && p.color_format == LUCID_COLOR_RGBA32F;
	const bool opacity_grads = p.dtri_opacity && p.tri_opacity;
	double acc64[3] = {0.0, 0.0, 0.0}, T64 = 1.0;
	float T = 1.0f;
	for(uint32_t j = 0; j < cnt; j++) {
		const uint32_t tri = p.grad_tris[off + j];
		if(tri >= 2u * uint32_t(p.max_visible_quads))
			continue; // only after a device error (the frame's lucid_info has it)
		const FragmentShade fs = shadeFragmentFull(p, tri, fragmentDepth(p, tri, x, y), x, y);
		const float4 c = fs.col;
		const float a = c.w;
		const float ca[3] = {c.x * a, c.y * a, c.z * a};
		const float cc[3] = {c.x, c.y, c.z};
		const double inv = 1.0 - double(a); // exact: a has a 24-bit mantissa
		const double rinv = inv != 0.0 ? 1.0 / inv : 0.0;
		double da = 0.0;
		float dc[3];
		for(int ch = 0; ch < 3; ch++) {
			acc64[ch] += double(ca[ch]) * T64;
			const double behind = c64[ch] - acc64[ch];
			dc[ch] = float(double(grad[ch]) * double(a) * T64);
			da += double(grad[ch]) * (double(cc[ch]) * T64 - behind * rinv);
		}
		T64 *= inv;
		if(vertex_grads && fs.has_vc) {
			// one vector reduction per vertex (RGBA rows are 16-byte aligned)
			const float dalpha = float(da) * fs.opacity;
			for(int k = 0; k < 3; k++)
				atomicAdd(reinterpret_cast<float4*>(p.dvertex_rgba) + fs.vid[k],
						  make_float4(fs.inst.x * fs.wgt[k] * dc[0], fs.inst.y * fs.wgt[k] * dc[1],
									  fs.inst.z * fs.wgt[k] * dc[2], fs.inst.w * fs.wgt[k] * dalpha));
		}
		if(opacity_grads)
			atomicAdd(p.dtri_opacity + fs.prim, float(da) * fs.alpha_pre);
		T = T * (1.0f - a);
		if(T == 0.0f)
			break;
	}
}

void launchBlendPixels(const FrameParams& p, cudaStream_t stream) {
	const dim3 block(kGradTileX, kGradTileY);
	const dim3 grid((p.width + kGradTileX - 1) / kGradTileX, (p.height + kGradTileY - 1) / kGradTileY);
	blendPixelsKernel<<<grid, block, 0, stream>>>(p);
}

void launchGradColor(const FrameParams& p, cudaStream_t stream) {
	const dim3 block(kGradTileX, kGradTileY);
	const dim3 grid((p.width + kGradTileX - 1) / kGradTileX, (p.height + kGradTileY - 1) / kGradTileY);
	gradColorKernel<<<grid, block, 0, stream>>>(p);
}

void launchGradBackward(const FrameParams& p, cudaStream_t stream) {
	const dim3 block(kGradTileX, kGradTileY);
	const dim3 grid((p.width + kGradTileX - 1) / kGradTileX, (p.height + kGradTileY - 1) / kGradTileY);
	gradBackwardKernel<<<grid, block, 0, stream>>>(p);
}

} // namespace lucid
