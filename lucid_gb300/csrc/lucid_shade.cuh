// Fragment shading shared by the raster pass and the gradient kernels: both must produce the
// same FP32 colour for a fragment, so there is one definition.
#pragma once

#include "lucid_common.cuh"

namespace lucid {

// Fragment colour (shading.glsl:107-165 without lighting/texturing; exact-mode FP32 colours).
__device__ __forceinline__ float4 shadeFragment(const FrameParams& p, uint32_t tri, float inv_ray_pos,
												int px, int py) {
	uint4 b0r = __ldg(p.tri_bary + size_t(tri) * 2);
	uint4 b1r = __ldg(p.tri_bary + size_t(tri) * 2 + 1);
	uint32_t fid = __ldg(&p.tri_depth[tri].w);
	float fx = float(px), fy = float(py);
	float ray_pos = 1.0f / inv_ray_pos;
	float e0 = bitsf(b0r.x) * fx + (bitsf(b0r.y) * fy + bitsf(b0r.z));
	float e1 = bitsf(b1r.x) * fx + (bitsf(b1r.y) * fy + bitsf(b1r.z));
	float b0 = e0 * ray_pos, b1 = e1 * ray_pos;
	b0 = b0 - bitsf(b0r.w);
	b1 = b1 - bitsf(b1r.w);
	uint32_t flags = fid & 0xffffu, inst = fid >> 16;
	float4 col = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
	if((flags & LUCID_INST_HAS_COLOR) && p.instance_colors)
		col = decodeRGBA8(__ldg(p.instance_colors + inst));
	if(flags & LUCID_INST_HAS_VERTEX_COLORS) {
		uint32_t quad = tri >> 1, second = tri & 1;
		uint4 qv = __ldg(p.quad_verts + quad);
		uint32_t v1 = second ? qv.z : qv.y, v2 = second ? qv.w : qv.z;
		float4 c0, c1, c2;
		if(p.color_format == LUCID_COLOR_RGBA8) {
			uint4 qc = __ldg(p.quad_colors + quad);
			c0 = decodeRGBA8(qc.x);
			c1 = decodeRGBA8(second ? qc.z : qc.y);
			c2 = decodeRGBA8(second ? qc.w : qc.z);
		} else if(p.color_format == LUCID_COLOR_RGBA16F) {
			const uint2* hc = reinterpret_cast<const uint2*>(p.colors);
			uint2 h0 = __ldg(hc + qv.x), h1 = __ldg(hc + v1), h2 = __ldg(hc + v2);
			auto cvt = [](uint2 h) {
				__half2 a = *reinterpret_cast<__half2*>(&h.x), b = *reinterpret_cast<__half2*>(&h.y);
				float2 fa = __half22float2(a), fb = __half22float2(b);
				return make_float4(fa.x, fa.y, fb.x, fb.y);
			};
			c0 = cvt(h0), c1 = cvt(h1), c2 = cvt(h2);
		} else {
			const float4* fc = reinterpret_cast<const float4*>(p.colors);
			c0 = __ldg(fc + qv.x), c1 = __ldg(fc + v1), c2 = __ldg(fc + v2);
		}
		float w = (1.0f - b0) - b1;
		col.x = col.x * (w * c0.x + (b0 * c1.x + b1 * c2.x));
		col.y = col.y * (w * c0.y + (b0 * c1.y + b1 * c2.y));
		col.z = col.z * (w * c0.z + (b0 * c1.z + b1 * c2.z));
		col.w = col.w * (w * c0.w + (b0 * c1.w + b1 * c2.w));
	}
	if(p.tri_opacity) {
		uint32_t prim = __ldg(p.quad_source + (tri >> 1)) * 2 + (tri & 1);
		col.w = col.w * __ldg(p.tri_opacity + prim);
	}
	return col;
}

// shadeFragment with everything the backward pass needs to route gradients to the vertex
// colours and the triangle opacity (same float operations, so the same colour).
struct FragmentShade {
	float4 col;           // colour used by the blend (alpha includes the opacity)
	float4 inst;          // instance colour factor
	float wgt[3];         // barycentric weights of the three vertices
	uint32_t vid[3];      // vertex ids
	float opacity;        // per-triangle opacity factor (1 if none)
	float alpha_pre;      // alpha before the opacity factor
	uint32_t prim;
	bool has_vc;
};

__device__ __forceinline__ FragmentShade shadeFragmentFull(const FrameParams& p, uint32_t tri,
														   float inv_ray_pos, int px, int py) {
	FragmentShade f;
	uint4 b0r = __ldg(p.tri_bary + size_t(tri) * 2);
	uint4 b1r = __ldg(p.tri_bary + size_t(tri) * 2 + 1);
	uint32_t fid = __ldg(&p.tri_depth[tri].w);
	float fx = float(px), fy = float(py);
	float ray_pos = 1.0f / inv_ray_pos;
	float e0 = bitsf(b0r.x) * fx + (bitsf(b0r.y) * fy + bitsf(b0r.z));
	float e1 = bitsf(b1r.x) * fx + (bitsf(b1r.y) * fy + bitsf(b1r.z));
	float b0 = e0 * ray_pos, b1 = e1 * ray_pos;
	b0 = b0 - bitsf(b0r.w);
	b1 = b1 - bitsf(b1r.w);
	uint32_t flags = fid & 0xffffu, inst = fid >> 16;
	f.inst = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
	if((flags & LUCID_INST_HAS_COLOR) && p.instance_colors)
		f.inst = decodeRGBA8(__ldg(p.instance_colors + inst));
	f.col = f.inst;
	float w = (1.0f - b0) - b1;
	f.wgt[0] = w, f.wgt[1] = b0, f.wgt[2] = b1;
	uint32_t quad = tri >> 1, second = tri & 1;
	uint4 qv = __ldg(p.quad_verts + quad);
	f.vid[0] = qv.x, f.vid[1] = second ? qv.z : qv.y, f.vid[2] = second ? qv.w : qv.z;
	f.has_vc = (flags & LUCID_INST_HAS_VERTEX_COLORS) != 0;
	if(f.has_vc) {
		float4 c0, c1, c2;
		if(p.color_format == LUCID_COLOR_RGBA8) {
			uint4 qc = __ldg(p.quad_colors + quad);
			c0 = decodeRGBA8(qc.x);
			c1 = decodeRGBA8(second ? qc.z : qc.y);
			c2 = decodeRGBA8(second ? qc.w : qc.z);
		} else if(p.color_format == LUCID_COLOR_RGBA16F) {
			const uint2* hc = reinterpret_cast<const uint2*>(p.colors);
			uint2 h0 = __ldg(hc + f.vid[0]), h1 = __ldg(hc + f.vid[1]), h2 = __ldg(hc + f.vid[2]);
			auto cvt = [](uint2 h) {
				__half2 a = *reinterpret_cast<__half2*>(&h.x), b = *reinterpret_cast<__half2*>(&h.y);
				float2 fa = __half22float2(a), fb = __half22float2(b);
				return make_float4(fa.x, fa.y, fb.x, fb.y);
			};
			c0 = cvt(h0), c1 = cvt(h1), c2 = cvt(h2);
		} else {
			const float4* fc = reinterpret_cast<const float4*>(p.colors);
			c0 = __ldg(fc + f.vid[0]), c1 = __ldg(fc + f.vid[1]), c2 = __ldg(fc + f.vid[2]);
		}
		f.col.x = f.col.x * (w * c0.x + (b0 * c1.x + b1 * c2.x));
		f.col.y = f.col.y * (w * c0.y + (b0 * c1.y + b1 * c2.y));
		f.col.z = f.col.z * (w * c0.z + (b0 * c1.z + b1 * c2.z));
		f.col.w = f.col.w * (w * c0.w + (b0 * c1.w + b1 * c2.w));
	}
	f.alpha_pre = f.col.w;
	f.opacity = 1.0f;
	f.prim = __ldg(p.quad_source + quad) * 2 + second;
	if(p.tri_opacity) {
		f.opacity = __ldg(p.tri_opacity + f.prim);
		f.col.w = f.col.w * f.opacity;
	}
	return f;
}

// Depth (inv_ray_pos) of a triangle's plane at pixel (px, py), evaluated as the raster's
// fragment keys are (shading.glsl:116): dx * px + (dy * py + dz).
__device__ __forceinline__ float fragmentDepth(const FrameParams& p, uint32_t tri, int px, int py) {
	uint4 d = __ldg(p.tri_depth + tri);
	float ty = bitsf(d.y) * float(py) + bitsf(d.z);
	return bitsf(d.x) * float(px) + ty;
}

} // namespace lucid
