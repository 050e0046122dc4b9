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

// ---------------------------------------------------------------------------------------------
// Reference-order shading (shadeSample with lighting, shading.glsl:107-184)

// x^y for finite x > 0 as exp2(y * log2(x)): log2 of the mantissa m in [sqrt(1/2), sqrt(2)) from
// the series 2 atanh(t) = ln(m), t = (m - 1) / (m + 1), up to t^13; 2^f, f in [0, 1), from the
// Taylor series of e^(f ln 2) up to degree 10. Every operation rounds separately (no FMA), so
// the result is the same on every IEEE single-precision implementation that runs these steps.
__device__ __forceinline__ float refPow(float x, float y) {
	if(x != x)
		return x;
	if(x <= 0.0f)
		return x == 0.0f ? 0.0f : __int_as_float(0x7fc00000);
	if(x == __int_as_float(0x7f800000))
		return y > 0.0f ? x : 0.0f;
	int e = 0;
	uint32_t b = fbits(x);
	if(((b >> 23) & 0xffu) == 0u) { // subnormal
		x = x * 8388608.0f;
		b = fbits(x);
		e = -23;
	}
	e += int((b >> 23) & 0xffu) - 127;
	float m = bitsf((b & 0x7fffffu) | 0x3f800000u);
	if(m > 0x1.6a09e6p+0f) {
		m = m * 0.5f;
		e = e + 1;
	}
	const float t = (m - 1.0f) / (m + 1.0f);
	const float t2 = t * t;
	float sr = 0x1.3b13b2p-4f;      // 1/13
	sr = sr * t2 + 0x1.745d18p-4f; // 1/11
	sr = sr * t2 + 0x1.c71c72p-4f; // 1/9
	sr = sr * t2 + 0x1.24924ap-3f; // 1/7
	sr = sr * t2 + 0x1.99999ap-3f; // 1/5
	sr = sr * t2 + 0x1.555556p-2f; // 1/3
	sr = sr * t2 + 1.0f;
	const float ln_m = (2.0f * t) * sr;
	const float l2 = float(e) + ln_m * 0x1.715476p+0f; // 1/ln 2
	const float z = y * l2;
	if(z >= 128.0f)
		return __int_as_float(0x7f800000);
	if(z < -149.0f)
		return 0.0f;
	const float k = floorf(z);
	const float u = (z - k) * 0x1.62e43p-1f; // ln 2
	float pe = 0x1.27e4fcp-22f;    // 1/10!
	pe = pe * u + 0x1.71de3ap-19f; // 1/9!
	pe = pe * u + 0x1.a01a02p-16f; // 1/8!
	pe = pe * u + 0x1.a01a02p-13f; // 1/7!
	pe = pe * u + 0x1.6c16c2p-10f; // 1/6!
	pe = pe * u + 0x1.111112p-7f;  // 1/5!
	pe = pe * u + 0x1.555556p-5f;  // 1/4!
	pe = pe * u + 0x1.555556p-3f;  // 1/3!
	pe = pe * u + 0.5f;
	pe = pe * u + 1.0f;
	pe = pe * u + 1.0f;
	int ki = int(k);
	if(ki < -126) { // scale in two steps to stay within normal exponents
		pe = pe * bitsf(uint32_t(ki + 126 + 127) << 23);
		ki = -126;
	}
	return pe * bitsf(uint32_t(ki + 127) << 23);
}

__device__ __forceinline__ float saturatef(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }

// RGBA8 sample colour (0 when alpha is 0) and depth of tri `tri` at pixel (px, py): the
// exact mode's colour, then the flat tri normal (funcs.glsl:61-66), sun light and
// finalShading with sRGB conversions (funcs.glsl:153-164, 261-271), encodeRGBA8
// (funcs.glsl:118-121).
__device__ __forceinline__ uint32_t shadeSampleRef(const FrameParams& p, uint32_t tri, int px, int py,
												   float& depth) {
	const float inv_ray_pos = fragmentDepth(p, tri, px, py);
	depth = inv_ray_pos;
	float4 c = shadeFragment(p, tri, inv_ray_pos, px, py);
	if(c.w == 0.0f)
		return 0u;
	const lucid_lighting& L = p.cfg.lighting;
	const uint32_t n = __ldg(p.tri_normals + tri);
	const float s511 = 0x1.00804p-9f; // 1/511
	const float nx = (float((n >> 0) & 0x3ffu) - 512.0f) * s511;
	const float ny = (float((n >> 10) & 0x3ffu) - 512.0f) * s511;
	const float nz = (float((n >> 20) & 0x3ffu) - 512.0f) * s511;
	const float dn = (-L.sun_dir[0]) * nx + (-L.sun_dir[1]) * ny + (-L.sun_dir[2]) * nz;
	const float light = fmaxf(0.0f, dn * 0x1.666666p-1f + 0x1.333334p-2f); // * 0.7 + 0.3
	float rgb[3] = {c.x, c.y, c.z};
	for(int ch = 0; ch < 3; ch++) {
		const float cv = rgb[ch];
		const float lin = cv < 0x1.4b5dccp-5f ? 0x1.3d0722p-4f * cv // 0.04045, 1/12.92
											  : refPow((cv + 0x1.c28f5cp-5f) * 0x1.e54edep-1f, 0x1.333334p+1f);
		const float amb = L.ambient_color[ch] * L.ambient_power;
		const float dif = (L.sun_color[ch] * L.sun_power) * light;
		const float v = lin * (amb + dif);
		const float sr = v < 0x1.9a5c38p-9f ? 0x1.9d70a4p+3f * v // 0.0031308, 12.92
											: 0x1.0e147ap+0f * refPow(v, 0x1.aaaaaap-2f) - 0x1.c28f5cp-5f;
		rgb[ch] = saturatef(sr);
	}
	return f2u(rgb[0] * 255.0f) | (f2u(rgb[1] * 255.0f) << 8) | (f2u(rgb[2] * 255.0f) << 16) |
		   (f2u(c.w * 255.0f) << 24);
}

} // namespace lucid
