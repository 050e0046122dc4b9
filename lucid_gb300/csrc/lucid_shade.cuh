// Fragment shading shared by the raster pass, the pixel-parallel kernels and the
// reference-order mode: every path must produce the same FP32 colour for a fragment, so there is
// one definition (shading.glsl:107-184), textures included.
#pragma once

#include "lucid_common.cuh"

namespace lucid {

// log2(x) for finite x > 0: exponent plus the series 2 atanh(t) = ln(m), t = (m - 1) / (m + 1),
// on the mantissa m in [sqrt(1/2), sqrt(2)) up to t^13. Every operation rounds separately (no
// FMA), so the result is the same on every IEEE single-precision implementation that runs these
// steps. 0 gives -inf, +inf gives +inf, negative or NaN input NaN.
__device__ __forceinline__ float seriesLog2(float x) {
	if(x != x || x < 0.0f)
		return __int_as_float(0x7fc00000);
	if(x == 0.0f)
		return __int_as_float(0xff800000);
	if(x == __int_as_float(0x7f800000))
		return x;
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
	return float(e) + ln_m * 0x1.715476p+0f; // 1/ln 2
}

// Texel (x, y) of mip level `level`, addressing repeated.
__device__ __forceinline__ float4 texLevelTexel(const lucid_texture& t, size_t off, int w, int h, int x, int y) {
	x = x < 0 ? x + w : (x >= w ? x - w : x);
	y = y < 0 ? y + h : (y >= h ? y - h : y);
	return decodeRGBA8(__ldg(t.texels + off + size_t(y) * w + x));
}

// Bilinear sample of one mip level at uv (repeat addressing, texel centres at half integers).
__device__ __forceinline__ float4 texSampleLevel(const lucid_texture& t, int level, float u, float v) {
	size_t off = 0;
	for(int l = 0; l < level; l++)
		off += size_t(max(1, t.width >> l)) * size_t(max(1, t.height >> l));
	const int w = max(1, t.width >> level), h = max(1, t.height >> level);
	u = u - floorf(u);
	v = v - floorf(v);
	if(u != u)
		u = 0.0f;
	if(v != v)
		v = 0.0f;
	const float fu = u * float(w) - 0.5f, fv = v * float(h) - 0.5f;
	const float xf = floorf(fu), yf = floorf(fv);
	const float a = fu - xf, b = fv - yf;
	const int x0 = int(xf), y0 = int(yf); // in [-1, size - 1]
	const float4 c00 = texLevelTexel(t, off, w, h, x0, y0), c10 = texLevelTexel(t, off, w, h, x0 + 1, y0);
	const float4 c01 = texLevelTexel(t, off, w, h, x0, y0 + 1), c11 = texLevelTexel(t, off, w, h, x0 + 1, y0 + 1);
	const float wa = (1.0f - a) * (1.0f - b), wb = a * (1.0f - b), wc = (1.0f - a) * b, wd = a * b;
	return make_float4(((c00.x * wa + c10.x * wb) + c01.x * wc) + c11.x * wd,
					   ((c00.y * wa + c10.y * wb) + c01.y * wc) + c11.y * wd,
					   ((c00.z * wa + c10.z * wb) + c01.z * wc) + c11.z * wd,
					   ((c00.w * wa + c10.w * wb) + c01.w * wc) + c11.w * wd);
}

// textureGrad with a trilinear, repeat-addressed sampler (the reference's sampler is trilinear
// with 16x anisotropy, src/lucid_base.h:30; the anisotropic footprint is the hardware's own and
// is not modelled): level of detail log2(max(|d uv/dx|, |d uv/dy|) in texels), clamped to the
// mip chain; bilinear samples of the two nearest levels blended by the fraction.
__device__ __forceinline__ float4 texSampleGrad(const lucid_texture& t, float u, float v, float dxu, float dxv,
												 float dyu, float dyv) {
	if(!t.texels)
		return make_float4(1.0f, 1.0f, 1.0f, 1.0f);
	const float W = float(t.width), H = float(t.height);
	const float ax = dxu * W, ay = dxv * H, bx = dyu * W, by = dyv * H;
	const float rho = fmaxf(sqrtf(ax * ax + ay * ay), sqrtf(bx * bx + by * by));
	float lambda = seriesLog2(rho);
	if(!(lambda > 0.0f))
		lambda = 0.0f;
	lambda = fminf(lambda, float(t.num_levels - 1));
	const float lf = floorf(lambda);
	const int l0 = int(lf);
	const float f = lambda - lf;
	float4 c = texSampleLevel(t, l0, u, v);
	if(f > 0.0f) {
		const float4 c1 = texSampleLevel(t, l0 + 1, u, v);
		const float g = 1.0f - f;
		c = make_float4(c.x * g + c1.x * f, c.y * g + c1.y * f, c.z * g + c1.z * f, c.w * g + c1.w * f);
	}
	return c;
}

// Everything shadeSample (shading.glsl:107-165) computes before lighting, in its float order.
struct ShadeCore {
	float4 col;      // colour with vertex colours and opacity (alpha includes the opacity)
	float4 factor;   // instance colour x texture colour: what multiplies the vertex colours
	float b0, b1;    // perspective-correct barycentrics of vertices 1 and 2
	float wgt;       // 1 - b0 - b1
	uint32_t vid[3]; // vertex ids
	uint32_t flags, inst;
	float opacity;   // per-triangle opacity factor (1 if none)
	float alpha_pre; // alpha before the opacity factor
	uint32_t prim;
};

// A tri's shading record (shadeRecWords(color_format) uint4 per tri, written by setup): the two barycentric
// plane records, then the vertex colours and instance flags | id << 16 (in c.w):
//   RGBA8:   c = (c0, c1, c2, flags_id)
//   RGBA16F: c = (c0.rg, c0.ba, c1.rg, flags_id), c2 = (c1.ba, c2.rg, c2.ba, 0) (IEEE halves)
//   RGBA32F: c = (0, 0, 0, flags_id); the colours are read from the inputs by vertex id
struct ShadeRec {
	uint4 b0, b1, c, c2;
};

__device__ __forceinline__ ShadeRec loadShadeRec(const FrameParams& p, uint32_t tri) {
	const bool half = p.color_format == LUCID_COLOR_RGBA16F;
	const uint4* rec = p.tri_shade + size_t(tri) * (half ? 4 : 3);
	ShadeRec r;
	r.b0 = __ldg(rec), r.b1 = __ldg(rec + 1), r.c = __ldg(rec + 2);
	r.c2 = half ? __ldg(rec + 3) : make_uint4(0u, 0u, 0u, 0u);
	return r;
}

__device__ __forceinline__ float4 halfRGBA(uint32_t rg, uint32_t ba) {
	__half2 a = *reinterpret_cast<__half2*>(&rg), b = *reinterpret_cast<__half2*>(&ba);
	float2 fa = __half22float2(a), fb = __half22float2(b);
	return make_float4(fa.x, fa.y, fb.x, fb.y);
}

__device__ __forceinline__ ShadeCore shadeCoreRec(const FrameParams& p, uint32_t tri, const ShadeRec& r,
												   float inv_ray_pos, int px, int py) {
	ShadeCore s;
	const uint4 b0r = r.b0, b1r = r.b1, crec = r.c;
	const uint32_t fid = crec.w;
	const float fx = float(px), fy = float(py);
	const float ray_pos = 1.0f / inv_ray_pos;
	const float e0 = bitsf(b0r.x) * fx + (bitsf(b0r.y) * fy + bitsf(b0r.z));
	const float e1 = bitsf(b1r.x) * fx + (bitsf(b1r.y) * fy + bitsf(b1r.z));
	const float braw0 = e0 * ray_pos, braw1 = e1 * ray_pos;
	const float b0 = braw0 - bitsf(b0r.w);
	const float b1 = braw1 - bitsf(b1r.w);
	s.b0 = b0, s.b1 = b1;
	s.flags = fid & 0xffffu, s.inst = fid >> 16;
	const uint32_t quad = tri >> 1, second = tri & 1;
	float4 col = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
	if((s.flags & LUCID_INST_HAS_COLOR) && p.instance_colors)
		col = decodeRGBA8(__ldg(p.instance_colors + s.inst));
	if(s.flags & LUCID_INST_HAS_ALBEDO_TEXTURE) {
		// shading.glsl:125-159: bary derivatives, texture coordinates, optional uv rect
		const uint4 d = __ldg(p.tri_depth + tri);
		const float ray_posx = 1.0f / (inv_ray_pos + bitsf(d.x));
		const float ray_posy = 1.0f / (inv_ray_pos + bitsf(d.y));
		const float bdx0 = (e0 + bitsf(b0r.x)) * ray_posx - braw0, bdx1 = (e1 + bitsf(b1r.x)) * ray_posx - braw1;
		const float bdy0 = (e0 + bitsf(b0r.y)) * ray_posy - braw0, bdy1 = (e1 + bitsf(b1r.y)) * ray_posy - braw1;
		const uint4 q0 = __ldg(p.quad_tex + size_t(quad) * 2), q1 = __ldg(p.quad_tex + size_t(quad) * 2 + 1);
		const float t0x = bitsf(q0.x), t0y = bitsf(q0.y);
		const float t1x = bitsf(second ? q1.x : q0.z), t1y = bitsf(second ? q1.y : q0.w);
		const float t2x = bitsf(second ? q1.z : q1.x), t2y = bitsf(second ? q1.w : q1.y);
		float u = b0 * t1x + (b1 * t2x + t0x), v = b0 * t1y + (b1 * t2y + t0y);
		float dxu = bdx0 * t1x + bdx1 * t2x, dxv = bdx0 * t1y + bdx1 * t2y;
		float dyu = bdy0 * t1x + bdy1 * t2x, dyv = bdy0 * t1y + bdy1 * t2y;
		if((s.flags & LUCID_INST_HAS_UV_RECT) && p.instance_uv_rects) {
			const float4 r = __ldg(p.instance_uv_rects + s.inst);
			u = r.z * (u - floorf(u)) + r.x;
			v = r.w * (v - floorf(v)) + r.y;
			dxu = dxu * r.z, dxv = dxv * r.w, dyu = dyu * r.z, dyv = dyv * r.w;
		}
		float4 tc;
		if(s.flags & LUCID_INST_TEX_OPAQUE) {
			tc = texSampleGrad(p.opaque_tex, u, v, dxu, dxv, dyu, dyv);
			tc.w = 1.0f;
		} else {
			tc = texSampleGrad(p.trans_tex, u, v, dxu, dxv, dyu, dyv);
		}
		col = make_float4(col.x * tc.x, col.y * tc.y, col.z * tc.z, col.w * tc.w);
	}
	s.factor = col;
	const float w = (1.0f - b0) - b1;
	s.wgt = w;
	s.vid[0] = s.vid[1] = s.vid[2] = 0u; // only read with FP32 vertex colours (gradients)
	if(s.flags & LUCID_INST_HAS_VERTEX_COLORS) {
		float4 c0, c1, c2;
		if(p.color_format == LUCID_COLOR_RGBA8) {
			c0 = decodeRGBA8(crec.x);
			c1 = decodeRGBA8(crec.y);
			c2 = decodeRGBA8(crec.z);
		} else if(p.color_format == LUCID_COLOR_RGBA16F) {
			c0 = halfRGBA(crec.x, crec.y);
			c1 = halfRGBA(crec.z, r.c2.x);
			c2 = halfRGBA(r.c2.y, r.c2.z);
		} else {
			const uint4 qv = __ldg(p.quad_verts + quad);
			s.vid[0] = qv.x, s.vid[1] = second ? qv.z : qv.y, s.vid[2] = second ? qv.w : qv.z;
			const float4* fc = reinterpret_cast<const float4*>(p.colors);
			c0 = __ldg(fc + s.vid[0]), c1 = __ldg(fc + s.vid[1]), c2 = __ldg(fc + s.vid[2]);
		}
		col.x = col.x * (w * c0.x + (b0 * c1.x + b1 * c2.x));
		col.y = col.y * (w * c0.y + (b0 * c1.y + b1 * c2.y));
		col.z = col.z * (w * c0.z + (b0 * c1.z + b1 * c2.z));
		col.w = col.w * (w * c0.w + (b0 * c1.w + b1 * c2.w));
	}
	s.alpha_pre = col.w;
	s.opacity = 1.0f;
	s.prim = 0u;
	if(p.tri_opacity) {
		s.prim = __ldg(p.quad_source + quad) * 2 + second;
		s.opacity = __ldg(p.tri_opacity + s.prim);
		col.w = col.w * s.opacity;
	}
	s.col = col;
	return s;
}

__device__ __forceinline__ ShadeCore shadeCore(const FrameParams& p, uint32_t tri, float inv_ray_pos, int px, int py) {
	return shadeCoreRec(p, tri, loadShadeRec(p, tri), inv_ray_pos, px, py);
}

// Fragment colour of the exact mode (shading.glsl:107-165 without lighting; FP32 colours).
__device__ __forceinline__ float4 shadeFragment(const FrameParams& p, uint32_t tri, float inv_ray_pos, int px,
												int py) {
	return shadeCore(p, tri, inv_ray_pos, px, py).col;
}

// shadeFragment with everything the backward pass needs to route gradients to the vertex
// colours and the triangle opacity (the same float operations, so the same colour).
struct FragmentShade {
	float4 col;      // colour used by the blend (alpha includes the opacity)
	float4 inst;     // instance colour x texture colour factor
	float wgt[3];    // barycentric weights of the three vertices
	uint32_t vid[3]; // vertex ids
	float opacity;   // per-triangle opacity factor (1 if none)
	float alpha_pre; // alpha before the opacity factor
	uint32_t prim;
	bool has_vc;
};

__device__ __forceinline__ FragmentShade shadeFragmentFull(const FrameParams& p, uint32_t tri, float inv_ray_pos,
														   int px, int py) {
	const ShadeCore c = shadeCore(p, tri, inv_ray_pos, px, py);
	FragmentShade f;
	f.col = c.col;
	f.inst = c.factor;
	f.wgt[0] = c.wgt, f.wgt[1] = c.b0, f.wgt[2] = c.b1;
	f.vid[0] = c.vid[0], f.vid[1] = c.vid[1], f.vid[2] = c.vid[2];
	f.opacity = c.opacity;
	f.alpha_pre = c.alpha_pre;
	f.prim = p.tri_opacity ? c.prim : __ldg(p.quad_source + (tri >> 1)) * 2 + (tri & 1);
	f.has_vc = (c.flags & LUCID_INST_HAS_VERTEX_COLORS) != 0;
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
	const float l2 = seriesLog2(x);
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

// funcs.glsl:61-66
__device__ __forceinline__ F3 decodeNormalUint(uint32_t n) {
	const float s511 = 0x1.00804p-9f; // 1/511
	return f3((float((n >> 0) & 0x3ffu) - 512.0f) * s511, (float((n >> 10) & 0x3ffu) - 512.0f) * s511,
			  (float((n >> 20) & 0x3ffu) - 512.0f) * s511);
}

// RGBA8 sample colour (0 when alpha is 0) and depth of tri `tri` at pixel (px, py): the
// exact mode's colour, then the flat tri normal (funcs.glsl:61-66), sun light and
// finalShading with sRGB conversions (funcs.glsl:153-164, 261-271), encodeRGBA8
// (funcs.glsl:118-121).
__device__ __forceinline__ uint32_t shadeSampleRef(const FrameParams& p, uint32_t tri, int px, int py,
												   float& depth) {
	const float inv_ray_pos = fragmentDepth(p, tri, px, py);
	depth = inv_ray_pos;
	const ShadeCore sc = shadeCore(p, tri, inv_ray_pos, px, py);
	const float4 c = sc.col;
	if(c.w == 0.0f)
		return 0u;
	const lucid_lighting& L = p.cfg.lighting;
	float nx, ny, nz;
	if((sc.flags & LUCID_INST_HAS_VERTEX_NORMALS) && p.normals) {
		// shading.glsl:168-174: normals interpolated with the perspective-correct barycentrics
		const uint4 qn = __ldg(p.quad_normals + (tri >> 1));
		const uint32_t second = tri & 1;
		const F3 n0 = decodeNormalUint(qn.x);
		const F3 n1 = decodeNormalUint(second ? qn.z : qn.y) - n0;
		const F3 n2 = decodeNormalUint(second ? qn.w : qn.z) - n0;
		nx = sc.b0 * n1.x + (sc.b1 * n2.x + n0.x);
		ny = sc.b0 * n1.y + (sc.b1 * n2.y + n0.y);
		nz = sc.b0 * n1.z + (sc.b1 * n2.z + n0.z);
	} else {
		const F3 n = decodeNormalUint(__ldg(p.tri_normals + tri));
		nx = n.x, ny = n.y, nz = n.z;
	}
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
