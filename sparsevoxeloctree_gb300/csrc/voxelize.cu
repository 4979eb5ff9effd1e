// voxelize.cu — triangles -> voxel fragments (replaces the reference's raster voxelizer:
// shader/voxelizer.{vert,geom,frag}, shader/voxelizer_conservative.geom, src/Voxelizer.cpp).
//
// Rule (identical to the oracle's restatement, see oracle/oracle.c):
//   coordinates snapped to 1/256 voxel (round to nearest even), dominant-axis projection
//   (shader/voxelizer.geom:27-36), a pixel is covered when each edge function's maximum over the
//   closed pixel square is >= 0 (the half-pixel dilation of shader/voxelizer_conservative.geom:46-58)
//   and the pixel lies in the triangle's pixel AABB (shader/voxelizer.frag:21-22); depth = floor of the
//   plane depth at the pixel centre, clamped to [0,R-1] and the triangle's depth range
//   (shader/voxelizer.frag:18-23); packing as shader/voxelizer.frag:40-42.
//
// GB300 design.  Coverage is computed per span (a row or column of the AABB, whichever makes fewer
// spans) from three exact interval bounds: a span costs three corrected float divisions whatever its
// length, or a few integer adds when the previous span of the same triangle is known (SpanWalk).  Triangle sizes span five orders of magnitude (a room wall covers 5e5 pixels, clutter ~10), so
// work is balanced at two granularities:
//   * small triangles (AABB <= kSmallArea pixels) are set up by one lane each, which walks the
//     triangle's spans; a warp writes its 32 small triangles' fragments together;
//   * large triangles are cut into units = (span, piece of <= kPiece pixels); units are flat work items
//     spread over the whole grid, so a wall becomes thousands of independent units.
// Passes (all stream-ordered, sizes stay on the device):
//   vox_classify_scan  per triangle: small -> fragment count, large -> unit count; both scanned with a
//                      single-pass decoupled look-back (small fragment offsets, large unit offsets);
//   vox_unit_scan      per unit: covered length, look-back scan -> fragment offset of every unit;
//   vox_emit           small triangles by warp, at their offsets;
//   vox_emit_units     units, 32 per warp, at their offsets (on a second stream beside vox_emit).
// Fragment order is deterministic: small triangles in input order, then large triangles in input order
// (spans, then pixels, in increasing order inside each).
#include <cstring>

#include "common.cuh"
#include "svo_internal.h"

namespace svo {

struct TriSetup {
	int32_t valid, axis, cols;
	int32_t u0, u1, v0, v1; // AABB in the span frame (u: inside a span, v: span index)
	int32_t z0, z1;
	int32_t gu[3], gv[3]; // edge k coefficients along U and V (sub-pixel units)
	int32_t pu[3], pv[3]; // origin vertex of edge k in (U, V)
	int64_t K, NU, NV, D; // depth numerator K - NU*u - NV*v over denominator D (> 0)
	uint32_t rgb;
	int32_t level;
};

SVO_DEV int32_t snap_coord(float p, float scale) {
	float q = p > 0.0f ? p : 0.0f; // also maps NaN to 0
	q = q < 1.0f ? q : 1.0f;
	return __float2int_rn(q * scale);
}

SVO_DEV uint32_t mean_color(uint32_t c0, uint32_t c1, uint32_t c2) {
	uint32_t out = 0;
#pragma unroll
	for (int ch = 0; ch < 3; ++ch) {
		uint32_t s = ((c0 >> (8 * ch)) & 0xffu) + ((c1 >> (8 * ch)) & 0xffu) + ((c2 >> (8 * ch)) & 0xffu);
		out |= (s / 3u) << (8 * ch);
	}
	return out;
}

SVO_DEV void tri_setup(const svo_triangle *__restrict__ tris, uint32_t t, uint32_t level, TriSetup &s) {
	const float4 *p = reinterpret_cast<const float4 *>(tris + t);
	float4 q0 = __ldg(p), q1 = __ldg(p + 1), q2 = __ldg(p + 2);
	const float v[9] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w, q2.x};
	s.rgb = mean_color(__float_as_uint(q2.y), __float_as_uint(q2.z), __float_as_uint(q2.w));
	s.level = (int32_t)level;
	const int32_t R = 1 << level;
	const float scale = (float)(256 << level);
	int32_t X[3], Y[3], Z[3];
#pragma unroll
	for (int k = 0; k < 3; ++k) {
		X[k] = snap_coord(v[3 * k], scale);
		Y[k] = snap_coord(v[3 * k + 1], scale);
		Z[k] = snap_coord(v[3 * k + 2], scale);
	}
	const int64_t e1x = X[1] - X[0], e1y = Y[1] - Y[0], e1z = Z[1] - Z[0];
	const int64_t e2x = X[2] - X[0], e2y = Y[2] - Y[0], e2z = Z[2] - Z[0];
	const int64_t nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
	s.valid = (nx | ny | nz) != 0;
	if (!s.valid) return;
	const int64_t ax = nx < 0 ? -nx : nx, ay = ny < 0 ? -ny : ny, az = nz < 0 ? -nz : nz;
	const int axis = (ax > ay && ax > az) ? 0 : (ay > az ? 1 : 2);
	s.axis = axis;
	// projected (a, b, depth): yzx / zxy / xyz (shader/voxelizer.geom:15-19)
	int32_t A[3], B[3], C[3];
#pragma unroll
	for (int k = 0; k < 3; ++k) {
		A[k] = axis == 0 ? Y[k] : (axis == 1 ? Z[k] : X[k]);
		B[k] = axis == 0 ? Z[k] : (axis == 1 ? X[k] : Y[k]);
		C[k] = axis == 0 ? X[k] : (axis == 1 ? Y[k] : Z[k]);
	}
	int64_t na = axis == 0 ? ny : (axis == 1 ? nz : nx);
	int64_t nb = axis == 0 ? nz : (axis == 1 ? nx : ny);
	int64_t nc = axis == 0 ? nx : (axis == 1 ? ny : nz);
	if (nc < 0) { // counter-clockwise in (a, b): swap vertices 1 and 2
		int32_t t0 = A[1], t1 = B[1], t2 = C[1];
		A[1] = A[2], B[1] = B[2], C[1] = C[2];
		A[2] = t0, B[2] = t1, C[2] = t2;
		na = -na, nb = -nb, nc = -nc;
	}
	const int32_t amin = min(A[0], min(A[1], A[2])), amax = max(A[0], max(A[1], A[2]));
	const int32_t bmin = min(B[0], min(B[1], B[2])), bmax = max(B[0], max(B[1], B[2]));
	const int32_t cmin = min(C[0], min(C[1], C[2])), cmax = max(C[0], max(C[1], C[2]));
	const int32_t i0 = clamp_i32(amin >> 8, 0, R - 1), i1 = clamp_i32(amax >> 8, 0, R - 1);
	const int32_t j0 = clamp_i32(bmin >> 8, 0, R - 1), j1 = clamp_i32(bmax >> 8, 0, R - 1);
	s.z0 = clamp_i32(cmin >> 8, 0, R - 1);
	s.z1 = clamp_i32(cmax >> 8, 0, R - 1);
	const int cols = (j1 - j0) > (i1 - i0);
	s.cols = cols;
	s.u0 = cols ? j0 : i0;
	s.u1 = cols ? j1 : i1;
	s.v0 = cols ? i0 : j0;
	s.v1 = cols ? i1 : j1;
#pragma unroll
	for (int k = 0; k < 3; ++k) {
		const int q = (k + 1) % 3;
		const int32_t ea = -(B[q] - B[k]), eb = A[q] - A[k];
		s.gu[k] = cols ? eb : ea;
		s.gv[k] = cols ? ea : eb;
		s.pu[k] = cols ? B[k] : A[k];
		s.pv[k] = cols ? A[k] : B[k];
	}
	// depth at the centre of pixel (i, j): floor((C0*nc - na*(256i+128-A0) - nb*(256j+128-B0)) / (256*nc))
	const int64_t nu = cols ? nb : na, nv = cols ? na : nb;
	const int64_t cu = cols ? B[0] : A[0], cv = cols ? A[0] : B[0];
	s.K = (int64_t)C[0] * nc - nu * (128 - cu) - nv * (128 - cv);
	s.NU = 256 * nu;
	s.NV = 256 * nv;
	s.D = 256 * nc;
}

// Covered interval [lo, hi] of span v (empty when lo > hi).
SVO_DEV void span_interval(const TriSetup &s, int32_t v, int32_t &lo, int32_t &hi) {
	const int32_t R = 1 << s.level;
	lo = s.u0;
	hi = s.u1;
#pragma unroll
	for (int k = 0; k < 3; ++k) {
		const int64_t g = s.gu[k], h = s.gv[k];
		const int64_t Ck = g * ((g > 0 ? 256 : 0) - s.pu[k]) + h * (256 * (int64_t)v + (h > 0 ? 256 : 0) - s.pv[k]);
		// 256 * g * u + Ck >= 0
		if (g > 0) {
			// ceil(-Ck / (256 g)) = -floor(Ck / (256 g)); exact where the bound falls in [0, R-1]
			const int64_t b = -floor_div_window(Ck, 256 * g, -(R - 1), 0);
			lo = max(lo, clamp_i32(b, -1, R));
		} else if (g < 0) {
			const int64_t b = floor_div_window(Ck, -256 * g, 0, R - 1);
			hi = min(hi, clamp_i32(b, -1, R));
		} else if (Ck < 0) {
			hi = lo - 1;
		}
	}
}

// floor(num / den) exactly, for den > 0 and |num / den| < 2^31: a float estimate, a second one from its
// remainder (within 1.001 of the remainder's quotient), and one final step.
SVO_DEV int64_t floor_div_exact(int64_t num, int64_t den) {
	const float fd = (float)den;
	int64_t q = (int64_t)__fdividef((float)num, fd); // within |num / den| * 2^-21 + 1 of the quotient
	int64_t r = num - q * den;
	const int64_t q2 = (int64_t)floorf(__fdividef((float)r, fd));
	q += q2;
	r -= q2 * den; // in [-0.001 den, 1.001 den)
	if (r < 0) {
		r += den;
		--q;
	} else if (r >= den) {
		r -= den;
		++q;
	}
	return q;
}

// The spans of a small triangle row by row.  Edge k bounds span v by floor(Ck(v) / den) with
// den = 256 |g| (span_interval), and Ck(v + 1) = Ck(v) + 256 h, so the quotient and remainder of row v + 1
// follow from row v's by integer adds: a row costs a few adds instead of three divisions, and its
// interval is span_interval's exactly.  An edge with g = 0 only empties rows on its outer side.  For a
// small triangle every Ck(v) / den lies within 2^29 (|g|, |h| <= 2^16, coordinates < 2^20).
struct SpanWalk {
	int32_t q[3], rem[3], dq[3], drem[3], den[3];
	int32_t kind[3]; // 1: lower bound -q, -1: upper bound q, 2 / -2 (g = 0): empty when q < 0 / q > 0
	int32_t u0, u1, R;
};

SVO_DEV void span_walk_init(const TriSetup &s, SpanWalk &w) {
	w.u0 = s.u0, w.u1 = s.u1, w.R = 1 << s.level;
#pragma unroll
	for (int k = 0; k < 3; ++k) {
		const int32_t g = s.gu[k], h = s.gv[k];
		if (g != 0) {
			const int32_t ag = g > 0 ? g : -g;
			const int64_t den = 256 * (int64_t)ag;
			const int64_t Ck = (int64_t)g * ((g > 0 ? 256 : 0) - s.pu[k]) +
			                   (int64_t)h * (256 * (int64_t)s.v0 + (h > 0 ? 256 : 0) - s.pv[k]);
			const int64_t q = floor_div_exact(Ck, den);
			int32_t dq = h / ag, dr = h - dq * ag; // floor(h / |g|) and 256 * (h mod |g|): the step 256 h
			if (dr < 0) dr += ag, --dq;
			w.kind[k] = g > 0 ? 1 : -1;
			w.q[k] = (int32_t)q, w.rem[k] = (int32_t)(Ck - q * den);
			w.dq[k] = dq, w.drem[k] = 256 * dr, w.den[k] = (int32_t)den;
		} else { // Ck = h * x with x = 256 v + (h > 0 ? 256 : 0) - pv
			w.kind[k] = h > 0 ? 2 : (h < 0 ? -2 : 0); // h = 0 too only for a degenerate (invalid) triangle
			w.q[k] = 256 * s.v0 + (h > 0 ? 256 : 0) - s.pv[k];
			w.rem[k] = 0, w.dq[k] = 256, w.drem[k] = 0, w.den[k] = 1;
		}
	}
}

// The interval [lo, hi] of the walk's current row (empty when lo > hi), then the walk moves to the next row.
SVO_DEV void span_walk_next(SpanWalk &w, int32_t &lo, int32_t &hi) {
	lo = w.u0, hi = w.u1;
	bool empty = false;
#pragma unroll
	for (int k = 0; k < 3; ++k) {
		const int32_t kd = w.kind[k], q = w.q[k];
		const int32_t b = min(max(kd == 1 ? -q : q, -1), w.R);
		if (kd == 1) lo = max(lo, b);
		if (kd == -1) hi = min(hi, b);
		empty |= (kd == 2 && q < 0) || (kd == -2 && q > 0);
		w.q[k] = q + w.dq[k];
		w.rem[k] += w.drem[k];
		if (w.rem[k] >= w.den[k]) w.rem[k] -= w.den[k], ++w.q[k];
	}
	if (empty) hi = lo - 1;
}

// AABB pixels up to which a triangle is small: set up once by one lane and emitted with its warp's other
// small triangles (256 measured fastest of 64..1024: fewer raster units, whose set-up repeats per span)
constexpr int kSmallArea = 256;
constexpr int kPiece = 256;     // pixels of a span one unit covers at most

SVO_DEV bool is_large(const TriSetup &s) {
	return s.valid && (int64_t)(s.u1 - s.u0 + 1) * (s.v1 - s.v0 + 1) > kSmallArea;
}

SVO_DEV uint32_t pieces_per_span(const TriSetup &s) { return (uint32_t)((s.u1 - s.u0) / kPiece + 1); }

SVO_DEV uint32_t unit_count(const TriSetup &s) { return (uint32_t)(s.v1 - s.v0 + 1) * pieces_per_span(s); }

// Unit `local` of a large triangle: its span v and the covered pixel interval [lo, hi] inside its piece.
SVO_DEV void unit_interval(const TriSetup &s, uint32_t local, int32_t &v, int32_t &lo, int32_t &hi) {
	const uint32_t pps = pieces_per_span(s);
	v = s.v0 + (int32_t)(local / pps);
	const int32_t p0 = s.u0 + (int32_t)(local % pps) * kPiece;
	span_interval(s, v, lo, hi);
	lo = max(lo, p0);
	hi = min(hi, p0 + kPiece - 1);
}

// Index of the last entry of the non-decreasing array a[0..n] that is <= x (a[0] = 0 <= x).
SVO_DEV uint32_t upper_index(const uint32_t *__restrict__ a, uint32_t n, uint32_t x) {
	uint32_t lo = 0, hi = n; // invariant a[lo] <= x < a[hi] (a[n] > x)
	while (hi - lo > 1) {
		const uint32_t mid = (lo + hi) >> 1;
		if (__ldg(a + mid) <= x)
			lo = mid;
		else
			hi = mid;
	}
	return lo;
}

// Warp-wide version for a warp-uniform x, with the invariant a[lo] <= x < a[hi]: each step probes 32
// evenly spaced entries at once and keeps the gap the ballot points at (4 dependent loads for n = 2^18).
SVO_DEV uint32_t warp_upper_index(const uint32_t *__restrict__ a, uint32_t lo, uint32_t hi, uint32_t x) {
	const uint32_t lane = lane_id();
	while (hi - lo > 1) {
		const uint32_t step = (hi - lo + 31) / 32;
		const uint32_t p = lo + lane * step;
		const bool le = p < hi && __ldg(a + p) <= x;
		const uint32_t c = __popc(__ballot_sync(kFullMask, le)); // >= 1: lane 0 probes lo
		lo += (c - 1) * step;
		hi = min(hi, lo + step);
	}
	return lo;
}

// Per-lane search inside [lo, hi) with a[lo] <= x < a[hi] (a short range that sits in L1).
SVO_DEV uint32_t upper_index_in(const uint32_t *__restrict__ a, uint32_t lo, uint32_t hi, uint32_t x) {
	while (hi - lo > 1) {
		const uint32_t mid = (lo + hi) >> 1;
		if (__ldg(a + mid) <= x)
			lo = mid;
		else
			hi = mid;
	}
	return lo;
}

// Triangle t of a batch's flat triangle index: its buffer, index in it, level and mesh.  A single
// voxelization (B = false) takes its one mesh by value and searches nothing.
template <bool B>
SVO_DEV void tri_of(const VoxBatch &vb, uint32_t t, const svo_triangle *&tris, uint32_t &local, uint32_t &level,
                    uint32_t &mi) {
	if constexpr (B) {
		mi = upper_index(vb.tri_base, vb.M, t);
		const VoxMesh vm = vb.table[mi];
		tris = vm.tris;
		local = t - __ldg(vb.tri_base + mi);
		level = vm.level;
	} else {
		mi = 0;
		tris = vb.one.tris;
		local = t;
		level = vb.one.level;
	}
}

// ---------------------------------------------------------------------------------------------------
constexpr int kTPB = 256;
// Items per thread of the scan tiles.  Larger tiles mean fewer look-backs (a tile waits for the prefix
// of the tiles before it) but more work per block: measured on the room, cluster and batch workloads,
// the count pass takes 2 triangles per thread below 2^20 triangles and 4 from there (kTile, the tile of
// the smaller form, sizes its descriptors), the unit scan 4 units per thread.
constexpr int kIPT = 2;
constexpr int kTile = kTPB * kIPT;
constexpr uint32_t kBigCountTris = 1u << 20;
constexpr int kUnitIPT = 4;
constexpr int kUnitTile = kTPB * kUnitIPT;

// Per triangle: small fragment count and large unit count, both exclusive-scanned.
//   small_off[t] = fragments of small triangles before t; small_off[n] = small total
//   unit_off[t]  = units of large triangles before t;    unit_off[n]  = unit total
// Persistent grid, tiles claimed in order by ticket, the two scans pipelined as in vox_unit_scan: a
// tile's aggregates are published once its counts are known, its look-backs and output follow after the
// block has counted its next tile.
template <bool B, int IPT>
__global__ void __launch_bounds__(kTPB) vox_classify_scan(VoxBatch vb, uint32_t n, VoxWorkspace w) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	constexpr int TILE = kTPB * IPT;
	__shared__ uint32_t s_tile;
	__shared__ uint32_t s_cnt[TILE];
	__shared__ uint32_t s_units[TILE];
	__shared__ unsigned long long s_warp[kTPB / 32 + 1];
	__shared__ unsigned long long s_prefix[2];
	const uint32_t ntiles = (uint32_t)(((uint64_t)n + TILE - 1) / TILE);
	// the pending tile: its aggregates published, its offsets not yet written
	uint32_t p_tile = 0xffffffffu, p_cnt[IPT], p_units[IPT];
	unsigned long long p_ec = 0, p_eu = 0, p_tc = 0, p_tu = 0;
	for (;;) {
		if (threadIdx.x == 0) s_tile = atomicAdd(&w.counters[kCtrTicketA], 1u);
		__syncthreads();
		const uint32_t tile = s_tile;
		__syncthreads();
		uint32_t cnt[IPT], unt[IPT];
		unsigned long long ec = 0, eu = 0, tc = 0, tu = 0;
		if (tile < ntiles) {
			const uint64_t base = (uint64_t)tile * TILE;
#pragma unroll 1
			for (int k = 0; k < IPT; ++k) {
				const uint64_t t = base + (uint64_t)k * kTPB + threadIdx.x;
				TriSetup s;
				s.valid = 0;
				if (t < n) {
					const svo_triangle *tp;
					uint32_t local, lvl, mi;
					tri_of<B>(vb, (uint32_t)t, tp, local, lvl, mi);
					tri_setup(tp, local, lvl, s);
				}
				const bool large = is_large(s);
				// small triangles: fragments = the covered lengths of their spans, walked row by row
				uint32_t frags = 0;
				if (s.valid && !large) {
					SpanWalk sw;
					span_walk_init(s, sw);
#pragma unroll 1
					for (int32_t v = s.v0; v <= s.v1; ++v) {
						int32_t lo, hi;
						span_walk_next(sw, lo, hi);
						frags += hi >= lo ? (uint32_t)(hi - lo + 1) : 0u;
					}
				}
				s_cnt[k * kTPB + threadIdx.x] = frags;
				s_units[k * kTPB + threadIdx.x] = large ? unit_count(s) : 0u;
			}
			__syncthreads();
			unsigned long long lc = 0, lu = 0;
#pragma unroll
			for (int k = 0; k < IPT; ++k) {
				cnt[k] = s_cnt[threadIdx.x * IPT + k];
				unt[k] = s_units[threadIdx.x * IPT + k];
				lc += cnt[k];
				lu += unt[k];
			}
			ec = block_exclusive_sum<unsigned long long, kTPB>(lc, s_warp, tc);
			eu = block_exclusive_sum<unsigned long long, kTPB>(lu, s_warp, tu);
			if (threadIdx.x == 0) {
				tile_publish_aggregate(w.descs, tile, 1u, tc);
				tile_publish_aggregate(w.descs2, tile, 1u, tu);
			}
		}
		if (p_tile != 0xffffffffu) { // the previous tile: look back (its predecessors are done), write
			if (threadIdx.x < 32) {
				const unsigned long long pc =
				    tile_lookback_warp(w.descs, p_tile, 1u, p_tc, &w.counters[kCtrStatus], false, true);
				const unsigned long long pu =
				    tile_lookback_warp(w.descs2, p_tile, 1u, p_tu, &w.counters[kCtrStatus], false, true);
				if (threadIdx.x == 0) s_prefix[0] = pc, s_prefix[1] = pu;
			}
			__syncthreads();
			const uint64_t base = (uint64_t)p_tile * TILE;
			unsigned long long rc = s_prefix[0] + p_ec, ru = s_prefix[1] + p_eu;
#pragma unroll
			for (int k = 0; k < IPT; ++k) {
				const uint64_t t = base + (uint64_t)threadIdx.x * IPT + k;
				if (t < n) {
					w.small_off[t] = rc;
					w.unit_off[t] = (uint32_t)ru;
				}
				rc += p_cnt[k];
				ru += p_units[k];
			}
			if (p_tile == ntiles - 1 && threadIdx.x == 0) {
				w.small_off[n] = s_prefix[0] + p_tc;
				const unsigned long long units = s_prefix[1] + p_tu;
				w.unit_off[n] = units > 0xffffffffull ? 0xffffffffu : (uint32_t)units;
				if (units > w.unit_cap) atomicOr(&w.counters[kCtrStatus], kStatusUnits);
			}
			__syncthreads();
		}
		if (tile >= ntiles) break;
		p_tile = tile, p_ec = ec, p_eu = eu, p_tc = tc, p_tu = tu;
#pragma unroll
		for (int k = 0; k < IPT; ++k) p_cnt[k] = cnt[k], p_units[k] = unt[k];
	}
}

// Per unit of a large triangle: covered length, scanned into unit_frag[u] (offset inside the large
// region); unit_frag[units] = large total.  Persistent grid: tiles claimed in order by ticket.  The scan
// is pipelined over a block's tiles: a tile publishes its aggregate as soon as its lengths are known,
// and its look-back and output come one tile later, after the block has measured its next tile, so a
// block does not idle at a barrier while its predecessors finish theirs.
template <bool B>
__global__ void __launch_bounds__(kTPB) vox_unit_scan(VoxBatch vb, uint32_t n, VoxWorkspace w) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	__shared__ uint32_t s_tile;
	__shared__ unsigned long long s_warp[kTPB / 32 + 1];
	__shared__ unsigned long long s_prefix;
	const uint32_t units = w.unit_off[n];
	if (units > w.unit_cap) return; // the host re-runs with a workspace sized for `units`
	const uint32_t ntiles = (units + kUnitTile - 1) / kUnitTile;
	uint32_t p_tile = 0xffffffffu, p_len[kUnitIPT]; // the pending tile: aggregate published, output not
	unsigned long long p_excl = 0, p_total = 0;
	for (;;) {
		if (threadIdx.x == 0) s_tile = atomicAdd(&w.counters[kCtrTicketB], 1u);
		__syncthreads();
		const uint32_t tile = s_tile;
		__syncthreads();
		uint32_t len[kUnitIPT];
		unsigned long long excl = 0, total = 0;
		if (tile < ntiles) {
			unsigned long long local = 0;
			// the warp's kUnitIPT * 32 consecutive units lie in triangles [t_first, t_last]
			const uint32_t u_first = tile * kUnitTile + (threadIdx.x & ~31u) * kUnitIPT;
			uint32_t t_first = 0, t_end = 0;
			if (u_first < units) {
				const uint32_t u_last = min(u_first + 32 * kUnitIPT - 1, units - 1);
				t_first = warp_upper_index(w.unit_off, 0, n, u_first);
				t_end = warp_upper_index(w.unit_off, t_first, n, u_last) + 1;
			}
#pragma unroll
			for (int k = 0; k < kUnitIPT; ++k) {
				const uint32_t u = tile * kUnitTile + threadIdx.x * kUnitIPT + k;
				len[k] = 0;
				if (u < units) {
					const uint32_t t = upper_index_in(w.unit_off, t_first, t_end, u);
					w.unit_tri[u] = t;
					TriSetup s;
					const svo_triangle *tp;
					uint32_t local_t, lvl, mi;
					tri_of<B>(vb, t, tp, local_t, lvl, mi);
					tri_setup(tp, local_t, lvl, s);
					int32_t v, lo, hi;
					unit_interval(s, u - w.unit_off[t], v, lo, hi);
					len[k] = hi >= lo ? (uint32_t)(hi - lo + 1) : 0u;
				}
				local += len[k];
			}
			excl = block_exclusive_sum<unsigned long long, kTPB>(local, s_warp, total);
			if (threadIdx.x == 0) tile_publish_aggregate(w.descs3, tile, 1u, total);
		}
		if (p_tile != 0xffffffffu) { // the previous tile: look back (its predecessors are done), write
			if (threadIdx.x < 32) {
				const unsigned long long p =
				    tile_lookback_warp(w.descs3, p_tile, 1u, p_total, &w.counters[kCtrStatus], false, true);
				if (threadIdx.x == 0) s_prefix = p;
			}
			__syncthreads();
			unsigned long long run = s_prefix + p_excl;
#pragma unroll
			for (int k = 0; k < kUnitIPT; ++k) {
				const uint32_t u = p_tile * kUnitTile + threadIdx.x * kUnitIPT + k;
				if (u < units) w.unit_frag[u] = run;
				run += p_len[k];
			}
			if (p_tile == ntiles - 1 && threadIdx.x == 0) w.unit_frag[units] = s_prefix + p_total;
			__syncthreads();
		}
		if (tile >= ntiles) break;
		p_tile = tile, p_excl = excl, p_total = total;
#pragma unroll
		for (int k = 0; k < kUnitIPT; ++k) p_len[k] = len[k];
	}
	if (ntiles == 0 && blockIdx.x == 0 && threadIdx.x == 0) w.unit_frag[0] = 0;
}

// Float value of num / den (den > 0, |num| <= den here) from the top 31 bits of both: 32-bit
// conversions only; relative error a few 2^-24.
SVO_DEV float ratio_f(int64_t num, int64_t den) {
	const uint64_t mag = (uint64_t)(num < 0 ? -num : num) | (uint64_t)den;
	const int sh = max(0, 33 - __clzll((long long)mag));
	return (float)(int32_t)(num >> sh) / (float)(int32_t)(den >> sh);
}

// The plane depth of a fragment (both emissions).  Pixel u = ua + k of span v lies at plane depth
// q0 + (r0 - k NU) / D, where num0 = K - NU ua - NV v, q0 = floor(num0 / D) and r0 = num0 - q0 D in
// [0, D) are taken once per span at an anchor pixel ua: a unit's first covered pixel (covered pixels lie
// within a voxel of the triangle's depth range, so the windowed division is exact there), or a small
// triangle's first bounding-box pixel u0 (exact division, carried from row to row).  t = fr0 - k fb
// (fr0 = r0 / D and fb = NU / D in float; |NU| <= D by the dominant axis) approximates (r0 - k NU) / D
// within 1e-4 for k < 256, so floor(t) is exact unless t lies within kDepthEps of an integer, where the
// exact int64 division decides.
constexpr float kDepthEps = 1.0f / 1024.0f;

SVO_DEV uint32_t field_of(int axis, int which) { return (uint32_t)((axis + which) % 3); } // 0 i, 1 j, 2 depth

// Emission of small triangles, 32 consecutive triangles per warp.  Each lane sets up its triangle,
// records it in shared memory and walks its rows (SpanWalk) into the warp's pool of kRowPool span rows:
// each row's first covered pixel and length, and its plane depth at the bounding box's first pixel in
// the form above.  Then the warp writes the group's fragments together: lane k takes fragments k, k+32,
// ... of the group (contiguous in the list: the small fragments are in triangle order), finds its row
// through the chunk's row map and packs the fragment from the row's depth (no division, outside the rare
// near-integer case), so every store instruction covers 256 contiguous bytes.  A small triangle has at
// most 16 spans (kMaxSmallSpans), so the pool holds every span of the warp.  (Evaluating the warp's rows
// one (triangle, row) pair per lane, three divisions per row, made this kernel 20-30% slower on
// small-triangle scenes; an int64 division per fragment cost another 6%.)  In a batch, mesh m's small
// fragments move up by its shift (the large fragments of earlier meshes).  Six blocks of four warps per
// SM: 80 registers.
constexpr int kEmitTPB = 128;

// A small triangle's record, as four 16-byte groups: the fragment loop reloads the first two when it
// moves to the next triangle, and reads the last two (the exact plane) only near integer depths.
struct __align__(16) SmallRec {
	float fb;             // NU / D
	uint32_t zr;          // z0 | z1 << 16: the depth range
	uint32_t rgbf;        // rgb | axis << 24 | cols << 26
	uint32_t rl;          // u0 | level << 16: the bounding box's first pixel along the spans
	uint64_t out;         // output position of its first fragment, minus that fragment's index in the group
	int32_t vadj;         // pooled row r is span v = r + vadj
	uint32_t spare;
	int64_t K, NU, NV, D; // plane depth (K - NU u - NV v) / D at the centre of pixel (u, v), D > 0
};
static_assert(sizeof(SmallRec) == 64, "four 16-byte groups");

// Span rows of a warp's 32 small triangles.  A span runs along the longer side of a triangle's
// bounding box (cols), so a small triangle (area <= kSmallArea pixels) has at most sqrt(kSmallArea) = 16
// spans, and the pool holds every span of the warp.
constexpr uint32_t kMaxSmallSpans = 16;
constexpr uint32_t kRowPool = 32 * kMaxSmallSpans;
constexpr uint32_t kFragChunk = 256; // fragments per pass of the fragment loop: 8 map entries per lane
static_assert(kMaxSmallSpans * kMaxSmallSpans >= (uint32_t)kSmallArea && (kMaxSmallSpans - 1) * (kMaxSmallSpans - 1) < (uint32_t)kSmallArea,
              "kMaxSmallSpans is the integer square root of kSmallArea");

// Fragment word of pixel (u, v), depth z of a triangle projected along `axis` with spans along `cols`
// (shader/voxelizer.frag:24,40-42: un-swizzle axis 0 -> u.zxy, 1 -> u.yzx, 2 -> u.xyz, then pack).
SVO_DEV uint64_t pack_fragment(uint32_t axis, uint32_t cols, uint32_t rgb, uint32_t u, uint32_t v, uint32_t z) {
	const uint32_t i = cols ? v : u, j = cols ? u : v;
	const uint32_t vx = axis == 0 ? z : (axis == 1 ? j : i);
	const uint32_t vy = axis == 0 ? i : (axis == 1 ? z : j);
	const uint32_t vz = axis == 0 ? j : (axis == 1 ? i : z);
	const uint32_t fx = vx | (vy << 12) | ((vz & 0xffu) << 24);
	const uint32_t fy = ((vz >> 8) << 28) | (rgb & 0xffffffu);
	return (uint64_t)fx | ((uint64_t)fy << 32);
}

static_assert(kFragChunk == 8 * 32, "a lane scans 8 map entries, one 16-byte group");

template <bool B>
__global__ void __launch_bounds__(kEmitTPB, 6) vox_emit(VoxBatch vb, uint32_t n, VoxWorkspace w,
                                                     uint64_t *__restrict__ frags, uint64_t capacity) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	__shared__ SmallRec s_rec[kEmitTPB];
	__shared__ uint32_t s_lq[kEmitTPB / 32][kRowPool];       // per pooled row: first pixel lo | q0 << 16 (int16 each)
	__shared__ float s_fr0[kEmitTPB / 32][kRowPool];         // per pooled row: fr0
	__shared__ uint16_t s_rcum[kEmitTPB / 32][kRowPool + 1]; // fragments of the group before each row
	__shared__ uint8_t s_rtri[kEmitTPB / 32][kRowPool];      // per pooled row: its triangle (lane)
	__shared__ __align__(16) uint16_t s_fmap[kEmitTPB / 32][kFragChunk]; // 1 + the row of each fragment of a chunk
	const uint32_t lane = lane_id(), wb = threadIdx.x & ~31u, wi = threadIdx.x >> 5;
	uint32_t *lq_of = s_lq[wi];
	float *fr0_of = s_fr0[wi];
	uint16_t *cum = s_rcum[wi];
	uint8_t *rtri = s_rtri[wi];
	uint16_t *fmap = s_fmap[wi];
	SmallRec *wrec = s_rec + wb;
	const uint4 *wrec4 = reinterpret_cast<const uint4 *>(wrec);
	const uint64_t warps = (uint64_t)gridDim.x * blockDim.x / 32;
	for (uint64_t g = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32; g * 32 < n; g += warps) {
		const uint64_t t = g * 32 + lane;
		uint32_t cnt = 0, rows = 0;
		SpanWalk sw;
		int64_t rd = 0, nv = 0, dd = 1; // plane depth at the row's pixel u0: quotient qd, remainder rd in [0, D)
		int32_t qd = 0;
		if (t < n) {
			uint64_t off = w.small_off[t];
			cnt = (uint32_t)(w.small_off[t + 1] - off);
			if (cnt) {
				const svo_triangle *tp;
				uint32_t local, lvl, mi;
				tri_of<B>(vb, (uint32_t)t, tp, local, lvl, mi);
				if (B) off += vb.shifts[2 * mi];
				TriSetup S;
				tri_setup(tp, local, lvl, S);
				if (!S.valid || is_large(S) || off + cnt > capacity) {
					cnt = 0;
				} else {
					SmallRec &r = s_rec[threadIdx.x];
					r.fb = ratio_f(S.NU, S.D);
					r.zr = (uint32_t)S.z0 | ((uint32_t)S.z1 << 16);
					r.rgbf = (S.rgb & 0xffffffu) | ((uint32_t)S.axis << 24) | ((uint32_t)S.cols << 26);
					r.rl = (uint32_t)S.u0 | ((uint32_t)S.level << 16);
					r.out = off;                    // - first fragment, below
					r.vadj = S.v0;                  // - first row, below
					r.K = S.K, r.NU = S.NU, r.NV = S.NV, r.D = S.D;
					rows = (uint32_t)(S.v1 - S.v0 + 1);
					span_walk_init(S, sw);
					const int64_t num = S.K - S.NU * S.u0 - S.NV * S.v0;
					qd = (int32_t)floor_div_exact(num, S.D);
					rd = num - (int64_t)qd * S.D, nv = S.NV, dd = S.D;
				}
			}
		}
		const uint32_t rincl = warp_inclusive_sum(rows), rfirst = rincl - rows;
		const uint32_t total_rows = __shfl_sync(kFullMask, rincl, 31);
		// each lane walks its triangle's rows into the pool: span, plane depth at pixel u0 (|NV| <= D, so
		// a row moves the quotient by at most one)
#pragma unroll 1
		for (uint32_t i = 0; i < rows; ++i) {
			const uint32_t r = rfirst + i;
			int32_t lo, hi;
			span_walk_next(sw, lo, hi);
			lq_of[r] = (uint32_t)(uint16_t)(int16_t)lo | ((uint32_t)qd << 16);
			fr0_of[r] = ratio_f(rd, dd);
			cum[r + 1] = (uint16_t)(hi >= lo ? hi - lo + 1 : 0); // the row's length, scanned below
			rtri[r] = (uint8_t)lane;
			rd -= nv;
			if (rd >= dd)
				rd -= dd, ++qd;
			else if (rd < 0)
				rd += dd, --qd;
		}
		__syncwarp();
		// row starts: an exclusive scan of the lengths over the rows (at most 32 x kSmallArea fragments)
		uint32_t carry = 0;
		for (uint32_t r0 = 0; r0 < total_rows; r0 += 32) {
			const uint32_t r = r0 + lane;
			const uint32_t len = r < total_rows ? cum[r + 1] : 0u;
			const uint32_t incl = warp_inclusive_sum(len) + carry;
			__syncwarp();
			if (r < total_rows) cum[r] = (uint16_t)(incl - len);
			carry = __shfl_sync(kFullMask, incl, 31);
			__syncwarp();
		}
		if (lane == 0) cum[total_rows] = (uint16_t)carry;
		__syncwarp();
		// a lane's fragments must be exactly its count (they are: the count pass walked the same spans)
		const uint32_t tstart = cum[rfirst], tend = cum[rincl];
		const bool ok = !rows || tend - tstart == cnt;
		if (__any_sync(kFullMask, !ok)) continue; // cannot happen; the group is left unwritten
		if (rows) {
			s_rec[threadIdx.x].out -= tstart;
			s_rec[threadIdx.x].vadj -= (int32_t)rfirst;
		}
		__syncwarp();
		// the group's fragments, kFragChunk at a time: each non-empty row marks its first fragment in the
		// chunk's map, a max scan over the map gives every fragment its row, and lane k takes fragments
		// k, k+32, ... of the chunk
		uint32_t row_carry = 0; // 1 + the last non-empty row starting before the chunk
		for (uint32_t c0 = 0; c0 < carry; c0 += kFragChunk) {
			reinterpret_cast<uint4 *>(fmap)[lane] = make_uint4(0u, 0u, 0u, 0u);
			__syncwarp();
			for (uint32_t r = lane; r < total_rows; r += 32) {
				const uint32_t st = cum[r];
				if (st >= c0 && st < c0 + kFragChunk && cum[r + 1] > st) fmap[st - c0] = (uint16_t)(r + 1);
			}
			__syncwarp();
			{ // inclusive max scan of the map: lane l holds entries 8l .. 8l+7
				const uint4 e = reinterpret_cast<const uint4 *>(fmap)[lane];
				uint32_t m8[8] = {e.x & 0xffffu, e.x >> 16, e.y & 0xffffu, e.y >> 16,
				                  e.z & 0xffffu, e.z >> 16, e.w & 0xffffu, e.w >> 16};
#pragma unroll
				for (int i = 1; i < 8; ++i) m8[i] = max(m8[i], m8[i - 1]);
				uint32_t m = m8[7];
#pragma unroll
				for (uint32_t d = 1; d < 32; d <<= 1) {
					const uint32_t o = __shfl_up_sync(kFullMask, m, d);
					if (lane >= d) m = max(m, o);
				}
				uint32_t before = __shfl_up_sync(kFullMask, m, 1);
				before = max(lane ? before : 0u, row_carry);
#pragma unroll
				for (int i = 0; i < 8; ++i) m8[i] = max(m8[i], before);
				reinterpret_cast<uint4 *>(fmap)[lane] = make_uint4(m8[0] | (m8[1] << 16), m8[2] | (m8[3] << 16),
				                                                   m8[4] | (m8[5] << 16), m8[6] | (m8[7] << 16));
				row_carry = max(row_carry, __shfl_sync(kFullMask, m, 31));
			}
			__syncwarp();
			const uint32_t cn = min((uint32_t)kFragChunk, carry - c0);
			for (uint32_t i = lane; i < cn; i += 32) {
				const uint32_t f = c0 + i, r = fmap[i] - 1u, jt = rtri[r];
				const uint4 g0 = wrec4[4 * jt], g1 = wrec4[4 * jt + 1];
				const float fb = __uint_as_float(g0.x);
				const uint32_t zr = g0.y, rgbf = g0.z, rl = g0.w;
				const uint64_t out = (uint64_t)g1.x | ((uint64_t)g1.y << 32);
				const int32_t vadj = (int32_t)g1.z;
				const uint32_t lq = lq_of[r];
				const int32_t u = (int32_t)(int16_t)(lq & 0xffffu) + (int32_t)(f - cum[r]), v = (int32_t)r + vadj;
				// the row's depth is taken at pixel u0 of the bounding box: k = u - u0 < 256
				const float tf = fmaf(-(float)(u - (int32_t)(rl & 0xffffu)), fb, fr0_of[r]);
				const float fl = floorf(tf);
				const float fr = tf - fl;
				int32_t z;
				if (fr >= kDepthEps && fr <= 1.0f - kDepthEps) {
					z = ((int32_t)lq >> 16) + (int32_t)fl;
				} else {
					const SmallRec &rec = wrec[jt];
					const int64_t num = rec.K - rec.NU * u - rec.NV * v;
					z = (int32_t)floor_div_window(num, rec.D, -2, (1 << (rl >> 16)) + 2);
				}
				const int32_t z0 = (int32_t)(zr & 0xffffu), z1 = (int32_t)(zr >> 16);
				const uint32_t zz = (uint32_t)(z < z0 ? z0 : (z > z1 ? z1 : z));
				frags[out + f] = pack_fragment((rgbf >> 24) & 3u, (rgbf >> 26) & 1u, rgbf, (uint32_t)u, (uint32_t)v, zz);
			}
			__syncwarp();
		}
	}
}

// One unit, prepared by the lane that owns it for the lanes that write its fragments.  Fragment k of
// the unit is pixel u = lo + k of span v, its depth in the row form above (q0, fr0, fb at the unit's
// first covered pixel).  The fragment words are base | u and z placed in their packed fields.
// The fields a lane reloads when it moves to another unit come first, as four 16-byte groups.
struct __align__(16) UnitRec {
	float fr0, fb;
	int32_t q0, lo;
	int32_t z0, z1, excl, R;   // R: resolution of the unit's mesh
	uint32_t ush, zsh;         // bit positions of u and z in the low fragment word
	uint32_t usplit, zsplit;   // all ones when u (z) is the z field, whose top 4 bits sit in the high word
	uint32_t base_lo, base_hi;
	uint64_t shift;            // output position of the unit's mesh's large region
	int64_t num0, nu, d;       // the exact division near integers
	uint64_t pad;
};

// Emission of large-triangle units, 32 consecutive units per warp.  Their fragments are contiguous in
// the output, so the warp writes them together: lane k takes fragments k, k+32, ... of the group (each
// store instruction covers 256 contiguous bytes), finds the unit holding its fragment and evaluates it
// from that unit's record.  In a batch, the units of one warp may belong to different meshes, each of
// whose large fragments start at its own shift.
template <bool B>
__global__ void __launch_bounds__(kTPB, 4) vox_emit_units(VoxBatch vb, uint32_t n, VoxWorkspace w,
                                                       uint64_t *__restrict__ frags, uint64_t capacity) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	__shared__ UnitRec s_rec[kTPB];
	__shared__ uint32_t s_incl[kTPB];
	const uint32_t units = w.unit_off[n];
	if (units > w.unit_cap) return; // reported by the count; nothing sensible to emit
	const uint64_t small_total = w.small_off[n];
	const uint32_t lane = lane_id();
	const UnitRec *warp_rec = s_rec + (threadIdx.x & ~31u);
	const uint32_t *warp_incl = s_incl + (threadIdx.x & ~31u);
	const uint64_t warps = (uint64_t)gridDim.x * blockDim.x / 32;
	for (uint64_t g = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32; g * 32 < units; g += warps) {
		const uint64_t u = g * 32 + lane;
		uint32_t len = 0;
		if (u < units) {
			const uint32_t t = w.unit_tri[u];
			TriSetup S;
			const svo_triangle *tp;
			uint32_t local, lvl, mi;
			tri_of<B>(vb, t, tp, local, lvl, mi);
			tri_setup(tp, local, lvl, S);
			const int32_t R = 1 << lvl;
			int32_t v, lo, hi;
			unit_interval(S, (uint32_t)u - w.unit_off[t], v, lo, hi);
			if (hi >= lo) {
				len = (uint32_t)(hi - lo + 1);
				UnitRec &rec = s_rec[threadIdx.x];
				const int64_t num0 = S.K - S.NU * lo - S.NV * v;
				const int64_t q0 = floor_div_window(num0, S.D, -2, R + 2);
				rec.q0 = (int32_t)q0;
				rec.fr0 = ratio_f(num0 - q0 * S.D, S.D);
				rec.fb = ratio_f(S.NU, S.D);
				rec.lo = lo;
				rec.z0 = S.z0;
				rec.z1 = S.z1;
				rec.num0 = num0;
				rec.nu = S.NU;
				rec.d = S.D;
				rec.R = R;
				rec.shift = B ? vb.shifts[2 * mi + 1] : small_total;
				// coordinate fields: i -> (axis+1)%3, j -> (axis+2)%3, depth -> axis (0 x, 1 y, 2 z)
				const uint32_t fi = field_of(S.axis, 1), fj = field_of(S.axis, 2), fz = field_of(S.axis, 0);
				const uint32_t fu = S.cols ? fj : fi, fv = S.cols ? fi : fj;
				rec.ush = 12u * fu, rec.zsh = 12u * fz;
				rec.usplit = fu == 2u ? 0xffffffffu : 0u, rec.zsplit = fz == 2u ? 0xffffffffu : 0u;
				const uint32_t vv = (uint32_t)v;
				rec.base_lo = vv << (12u * fv);
				rec.base_hi = (S.rgb & 0xffffffu) | (fv == 2u ? (vv >> 8) << 28 : 0u);
			}
		}
		const uint32_t incl = warp_inclusive_sum(len);
		const uint32_t total = __shfl_sync(kFullMask, incl, 31);
		s_incl[threadIdx.x] = incl;
		s_rec[threadIdx.x].excl = (int32_t)(incl - len);
		__syncwarp();
		const uint64_t first = (uint64_t)w.unit_frag[g * 32];
		uint32_t j = 0, have = 32;
		uint64_t out0 = 0;
		int32_t k = 0, q0 = 0, lo = 0, z0 = 0, z1 = 0, R = 0;
		float kf = 0.0f, fr0 = 0.0f, fb = 0.0f;
		uint32_t ush = 0, zsh = 0, usplit = 0, zsplit = 0, base_lo = 0, base_hi = 0;
#pragma unroll 2
		for (uint32_t f = lane; f < total; f += 32) {
			while (warp_incl[j] <= f) ++j;
			if (j != have) { // the record's first 64 bytes in four vector loads
				const uint4 *rr = reinterpret_cast<const uint4 *>(warp_rec + j);
				const uint4 g0 = rr[0], g1 = rr[1], g2 = rr[2], g3 = rr[3];
				fr0 = __uint_as_float(g0.x), fb = __uint_as_float(g0.y), q0 = (int32_t)g0.z, lo = (int32_t)g0.w;
				z0 = (int32_t)g1.x, z1 = (int32_t)g1.y, R = (int32_t)g1.w;
				k = (int32_t)(f - g1.z);
				kf = (float)k;
				ush = g2.x, zsh = g2.y, usplit = g2.z, zsplit = g2.w;
				base_lo = g3.x, base_hi = g3.y;
				out0 = ((uint64_t)g3.z | ((uint64_t)g3.w << 32)) + first;
				have = j;
			} else {
				k += 32;
				kf += 32.0f;
			}
			const float tf = fmaf(-kf, fb, fr0);
			const float fl = floorf(tf);
			const float fr = tf - fl;
			int32_t z;
			if (fr >= kDepthEps && fr <= 1.0f - kDepthEps) {
				z = q0 + (int32_t)fl;
			} else {
				const UnitRec &rec = warp_rec[j];
				z = (int32_t)floor_div_window(rec.num0 - (int64_t)k * rec.nu, rec.d, -2, R + 2);
			}
			const uint32_t zz = (uint32_t)(z < z0 ? z0 : (z > z1 ? z1 : z)), uu = (uint32_t)(lo + k);
			const uint32_t flo = base_lo | (uu << ush) | (zz << zsh);
			const uint32_t fhi = base_hi | (((uu >> 8) << 28) & usplit) | (((zz >> 8) << 28) & zsplit);
			if (out0 + f < capacity) frags[out0 + f] = (uint64_t)flo | ((uint64_t)fhi << 32);
		}
		__syncwarp();
	}
}

// ---------------------------------------------------------------------------------------------------
// Workspace: small_off[n+1] u64 | unit_off[n+1] u32 | unit_frag[unit_cap+1] u64 | unit_tri[unit_cap+1] u32 |
// 3 descriptor arrays |
// counters.  unit_cap is a first guess; a larger unit total makes the count report it and the caller
// retries with vox_workspace_bytes(n, units).
uint64_t vox_default_unit_cap(uint32_t n) { return 2ull * n + 65536; }

static size_t tiles_for(uint64_t items, uint64_t tile = kTile) { return (size_t)((items + tile - 1) / tile + 1); }

size_t vox_workspace_bytes(uint32_t n, uint64_t unit_cap) {
	VoxWorkspace w;
	return vox_workspace_layout(nullptr, n, unit_cap, w);
}

size_t vox_workspace_layout(void *ws, uint32_t n, uint64_t unit_cap, VoxWorkspace &w) {
	char *p = (char *)ws;
	size_t off = 0;
	auto take = [&](size_t bytes) {
		char *q = p + off;
		off += align_up(bytes, 256);
		return q;
	};
	w.n = n;
	w.unit_cap = unit_cap;
	w.small_off = (uint64_t *)take(sizeof(uint64_t) * ((size_t)n + 1));
	w.unit_off = (uint32_t *)take(sizeof(uint32_t) * ((size_t)n + 1));
	w.unit_frag = (unsigned long long *)take(sizeof(unsigned long long) * (size_t)(unit_cap + 1));
	w.unit_tri = (uint32_t *)take(sizeof(uint32_t) * (size_t)(unit_cap + 1));
	const size_t t1 = tiles_for(n), t3 = tiles_for(unit_cap, kUnitTile);
	w.descs = (unsigned long long *)(p + off);
	w.desc_bytes = align_up((2 * t1 + t3) * sizeof(unsigned long long), 256);
	w.descs2 = w.descs + t1;
	w.descs3 = w.descs + 2 * t1;
	off += w.desc_bytes;
	w.counters = (uint32_t *)take(kCtrCount * sizeof(uint32_t));
	w.totals = (unsigned long long *)take(4 * sizeof(unsigned long long));
	return off;
}

static VoxBatch single_vox(const svo_triangle *tris, uint32_t level) {
	VoxBatch vb;
	memset(&vb, 0, sizeof(vb));
	vb.M = 1;
	vb.one.tris = tris;
	vb.one.level = level;
	return vb;
}

static cudaError_t clear_count_state(uint32_t n, const VoxWorkspace &w, cudaStream_t stream) {
	// the scan descriptors and the counters are adjacent in the layout: one memset
	cudaError_t e = cudaMemsetAsync(w.descs, 0, (size_t)((char *)(w.counters + kCtrCount) - (char *)w.descs), stream);
	if (e != cudaSuccess) return e;
	if (n == 0) {
		e = cudaMemsetAsync(w.small_off, 0, sizeof(uint64_t), stream);
		if (e == cudaSuccess) e = cudaMemsetAsync(w.unit_off, 0, sizeof(uint32_t), stream);
		if (e == cudaSuccess) e = cudaMemsetAsync(w.unit_frag, 0, sizeof(unsigned long long), stream);
	}
	return e;
}

template <bool B> static void launch_count(const VoxBatch &vb, uint32_t n, const VoxWorkspace &w, cudaStream_t stream) {
	const int sms = device_sm_count();
	if (n >= kBigCountTris)
		SVO_LAUNCH("vox_classify_scan", stream,
		           ::svo::launch_k(vox_classify_scan<B, 2 * kIPT>,
		                           std::min((n + 2 * kTile - 1) / (2 * kTile), resident_grid(vox_classify_scan<B, 2 * kIPT>, kTPB)),
		                           kTPB, 0, stream, vb, n, w););
	else
		SVO_LAUNCH("vox_classify_scan", stream,
		           ::svo::launch_k(vox_classify_scan<B, kIPT>,
		                           std::min((n + kTile - 1) / kTile, resident_grid(vox_classify_scan<B, kIPT>, kTPB)), kTPB, 0,
		                           stream, vb, n, w););
	SVO_LAUNCH("vox_unit_scan", stream, ::svo::launch_k(vox_unit_scan<B>, (uint32_t)sms * 4, kTPB, 0, stream, vb, n, w););
}

template <bool B>
static void launch_emit(const VoxBatch &vb, uint32_t n, uint32_t tune_level, const VoxWorkspace &w, uint64_t *frags,
                        uint64_t capacity, cudaStream_t stream, bool two_streams = true) {
	const int sms = device_sm_count();
	const uint32_t per_sm = (uint32_t)tune_value(kTuneEmitBlocks, tune_level, n);
	// the small triangles' and the units' fragments go to disjoint ranges: the two emissions run on two
	// streams, so each fills the SMs the other's tail leaves idle
	SideFork fork(stream, two_streams);
	cudaStream_t side = fork.side();
	SVO_LAUNCH("vox_emit", side,
	           ::svo::launch_k(vox_emit<B>, (uint32_t)sms * per_sm * (kTPB / kEmitTPB), kEmitTPB, 0, side, vb, n, w, frags, capacity););
	fork.mark_side(0);
	SVO_LAUNCH("vox_emit_units", stream,
	           ::svo::launch_k(vox_emit_units<B>, (uint32_t)sms * std::max(1u, per_sm / 2), kTPB, 0, stream, vb, n, w, frags, capacity););
	fork.main_waits(0);
}

cudaError_t vox_set_wait_fault(uint32_t limit, uint32_t withheld) { return set_wait_fault_here(limit, withheld); }

// Count, totals and emission of one mesh into an output buffer known in advance.  The small-triangle
// emission needs only the count pass's triangle offsets, so it starts on a second stream as soon as the
// count pass ends, beside the unit scan and the unit emission; the totals (read only after the call)
// follow it there once the unit scan is done.
cudaError_t vox_launch_count_emit(const svo_triangle *tris, uint32_t n, uint32_t level, const VoxWorkspace &w,
                                  uint64_t *frags, uint64_t capacity, cudaStream_t stream) {
	cudaError_t e = clear_count_state(n, w, stream);
	if (e != cudaSuccess) return e;
	if (n == 0) return vox_launch_totals(w, stream);
	const VoxBatch vb = single_vox(tris, level);
	const int sms = device_sm_count();
	if (n >= kBigCountTris)
		SVO_LAUNCH("vox_classify_scan", stream,
		           ::svo::launch_k(vox_classify_scan<false, 2 * kIPT>,
		                           std::min((n + 2 * kTile - 1) / (2 * kTile), resident_grid(vox_classify_scan<false, 2 * kIPT>, kTPB)),
		                           kTPB, 0, stream, vb, n, w););
	else
		SVO_LAUNCH("vox_classify_scan", stream,
		           ::svo::launch_k(vox_classify_scan<false, kIPT>,
		                           std::min((n + kTile - 1) / kTile, resident_grid(vox_classify_scan<false, kIPT>, kTPB)), kTPB, 0,
		                           stream, vb, n, w););
	const uint32_t per_sm = (uint32_t)tune_value(kTuneEmitBlocks, level, n);
	SideFork fork(stream, true);
	cudaStream_t side = fork.side();
	SVO_LAUNCH("vox_emit", side,
	           ::svo::launch_k(vox_emit<false>, (uint32_t)sms * per_sm * (kTPB / kEmitTPB), kEmitTPB, 0, side, vb, n, w, frags, capacity););
	SVO_LAUNCH("vox_unit_scan", stream, ::svo::launch_k(vox_unit_scan<false>, (uint32_t)sms * 4, kTPB, 0, stream, vb, n, w););
	fork.side_waits_main();
	e = vox_launch_totals(w, side);
	if (e != cudaSuccess) return e;
	fork.mark_side(0);
	SVO_LAUNCH("vox_emit_units", stream,
	           ::svo::launch_k(vox_emit_units<false>, (uint32_t)sms * std::max(1u, per_sm / 2), kTPB, 0, stream, vb, n, w, frags, capacity););
	fork.main_waits(0);
	return cudaGetLastError();
}

cudaError_t vox_launch_count(const svo_triangle *tris, uint32_t n, uint32_t level, const VoxWorkspace &w,
                             cudaStream_t stream) {
	cudaError_t e = clear_count_state(n, w, stream);
	if (e != cudaSuccess || n == 0) return e;
	launch_count<false>(single_vox(tris, level), n, w, stream);
	return cudaGetLastError();
}

cudaError_t vox_launch_emit(const svo_triangle *tris, uint32_t n, uint32_t level, const VoxWorkspace &w,
                            uint64_t *frags, uint64_t capacity, cudaStream_t stream, bool two_streams) {
	if (n == 0) return cudaSuccess;
	launch_emit<false>(single_vox(tris, level), n, level, w, frags, capacity, stream, two_streams);
	return cudaGetLastError();
}

__global__ void vox_totals(VoxWorkspace w) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	const uint32_t units = w.unit_off[w.n];
	const uint32_t status = w.counters[kCtrStatus];
	w.totals[0] = w.small_off[w.n] + ((status & kStatusUnits) ? 0ull : w.unit_frag[units]);
	w.totals[1] = units;
	w.totals[2] = status;
}

cudaError_t vox_launch_totals(const VoxWorkspace &w, cudaStream_t stream) {
	SVO_LAUNCH("vox_totals", stream, ::svo::launch_k(vox_totals, 1, 1, 0, stream, w););
	return cudaGetLastError();
}

cudaError_t vox_launch_count_batch(const VoxBatch &vb, uint32_t n, const VoxWorkspace &w, cudaStream_t stream) {
	cudaError_t e = clear_count_state(n, w, stream);
	if (e != cudaSuccess || n == 0) return e;
	launch_count<true>(vb, n, w, stream);
	return cudaGetLastError();
}

cudaError_t vox_launch_emit_batch(const VoxBatch &vb, uint32_t n, const VoxWorkspace &w, uint64_t *frags,
                                  uint64_t capacity, cudaStream_t stream) {
	if (n == 0) return cudaSuccess;
	launch_emit<true>(vb, n, vb.max_level, w, frags, capacity, stream);
	return cudaGetLastError();
}

// Per mesh m (triangles [T0, T1), units [U0, U1)): fragments = small + large, first fragment =
// small_off[T0] + unit_frag[U0] (everything of earlier meshes), small shift = unit_frag[U0] (large
// fragments of earlier meshes sit before its small ones), large shift = small_off[T1] (every small
// fragment up to the end of the mesh sits before its large ones).  Thread 0 also writes the totals.
__global__ void vox_batch_totals(VoxBatch vb, VoxWorkspace w) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	const uint32_t status = w.counters[kCtrStatus];
	const bool units_ok = !(status & kStatusUnits);
	for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < vb.M; m += gridDim.x * blockDim.x) {
		const uint32_t t0 = vb.tri_base[m], t1 = vb.tri_base[m + 1];
		const uint32_t u0 = w.unit_off[t0], u1 = w.unit_off[t1];
		const unsigned long long s0 = w.small_off[t0], s1 = w.small_off[t1];
		const unsigned long long f0 = units_ok ? w.unit_frag[u0] : 0ull, f1 = units_ok ? w.unit_frag[u1] : 0ull;
		vb.shifts[2 * m] = f0;
		vb.shifts[2 * m + 1] = s1;
		vb.mesh_out[4 * m] = (s1 - s0) + (f1 - f0);
		vb.mesh_out[4 * m + 1] = s0 + f0;
		vb.mesh_out[4 * m + 2] = u1 - u0;
		vb.mesh_out[4 * m + 3] = 0;
	}
	if (blockIdx.x == 0 && threadIdx.x == 0) {
		const uint32_t units = w.unit_off[w.n];
		w.totals[0] = w.small_off[w.n] + (units_ok ? w.unit_frag[units] : 0ull);
		w.totals[1] = units;
		w.totals[2] = status;
	}
}

cudaError_t vox_launch_batch_totals(const VoxBatch &vb, uint32_t n, const VoxWorkspace &w, cudaStream_t stream) {
	(void)n;
	SVO_LAUNCH("vox_totals", stream, ::svo::launch_k(vox_batch_totals, (vb.M + 127) / 128, 128, 0, stream, vb, w););
	return cudaGetLastError();
}

} // namespace svo
