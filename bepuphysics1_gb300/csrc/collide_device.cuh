// Device narrow phase: contact generation for box-box, box-sphere and
// sphere-sphere pairs and the manifold update that carries contacts and their
// warm-start impulses from one step to the next.
//
// The arithmetic restates, operation for operation, the reference's managed
// code path (the netstandard build compiles without ALLOWUNSAFE):
//   BoxBoxCollider.AreBoxesColliding (BoxBoxCollider.cs:1494-2388) with
//     GetEdgeEdgeContact (:2392-2698), GetFaceContacts (:3459-3487),
//     ClipFacesDirect (:4517-5278), PruneContactsMaxDistance (:3612-3700),
//     GetNearestFace (:6042-6178), ComputeIntersection (:6007-6040)
//   BoxSphereTester.AreShapesColliding (BoxSphereTester.cs:23-84)
//   SphereTester.AreSpheresColliding (SphereTester.cs:22-55)
//   BoxContactManifold.Update (BoxContactManifold.cs:122-196),
//   Box/SphereContactManifold.Update (:55-83) and the constraint's
//   AddContact / RemoveContact (ConvexContactManifoldConstraint.cs:117-155).
// One thread owns one manifold; candidate lists live in local arrays of eight
// (TinyStructList's capacity).  Built with -fmad=false like the rest of the
// library; (float)Math.Sqrt of a float is the IEEE float square root, and
// Vector3.Normalize's 1/Math.Sqrt stays in double.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "solver_device.cuh"

namespace bepugpu {
namespace nphase {

constexpr float kEps = 1e-7f;     // Toolbox.Epsilon
constexpr float kBigEps = 1e-5f;  // Toolbox.BigEpsilon

struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 mk(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator-(V3 a) { return mk(-a.x, -a.y, -a.z); }
__device__ __forceinline__ V3 scale(V3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float len2(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float comp(V3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
__device__ __forceinline__ float clampf(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Matrix3x3.CreateFromQuaternion (Matrix3x3.cs:1303-1328), as three rows.
__device__ __forceinline__ void Rows(float4 q, V3 r[3]) {
    float x2 = q.x + q.x, y2 = q.y + q.y, z2 = q.z + q.z;
    float XX = x2 * q.x, YY = y2 * q.y, ZZ = z2 * q.z;
    float XY = x2 * q.y, XZ = x2 * q.z, XW = x2 * q.w;
    float YZ = y2 * q.z, YW = y2 * q.w, ZW = z2 * q.w;
    r[0] = mk(1 - YY - ZZ, XY + ZW, XZ - YW);
    r[1] = mk(XY - ZW, 1 - XX - ZZ, YZ + XW);
    r[2] = mk(XZ + YW, YZ - XW, 1 - XX - YY);
}
// Matrix3x3.Transform (row vector times matrix) and TransformTranspose.
__device__ __forceinline__ V3 RowTimes(V3 v, const V3 r[3]) {
    return mk(v.x * r[0].x + v.y * r[1].x + v.z * r[2].x, v.x * r[0].y + v.y * r[1].y + v.z * r[2].y,
              v.x * r[0].z + v.y * r[1].z + v.z * r[2].z);
}
__device__ __forceinline__ V3 TimesRows(V3 v, const V3 r[3]) {
    return mk(v.x * r[0].x + v.y * r[0].y + v.z * r[0].z, v.x * r[1].x + v.y * r[1].y + v.z * r[1].z,
              v.x * r[2].x + v.y * r[2].y + v.z * r[2].z);
}
// Quaternion.Transform (Quaternion.cs).
__device__ __forceinline__ V3 QRot(V3 v, float4 r) {
    float3 o = QTransform(v.x, v.y, v.z, r);
    return mk(o.x, o.y, o.z);
}

// Candidate contacts (TinyStructList<BoxContactData>: eight entries, adds
// past eight dropped, RemoveAt shifts down).
struct Cands {
    V3 p[8];
    float d[8];
    int id[8];
    int n;
    __device__ __forceinline__ void add(V3 pos, float depth, int i) {
        if (n < 8) { p[n] = pos; d[n] = depth; id[n] = i; n++; }
    }
    __device__ __forceinline__ void removeAt(int i) {
        for (int k = i; k + 1 < n; k++) { p[k] = p[k + 1]; d[k] = d[k + 1]; id[k] = id[k + 1]; }
        n--;
    }
};

__device__ __forceinline__ int EdgeId(int a, int b) { return (a + 1) * 571 + (b + 1) * 577; }

// BoxBoxCollider.GetEdgeData: index bits pick the signs of the two axes other
// than `axis`; vertex ids are 4x + 2y + z with 1 on the positive side.
__device__ __forceinline__ void EdgeData(int index, int axis, V3 h, V3& s, V3& e, int& sId, int& eId) {
    const bool hi = (index >> 1) & 1, lo = index & 1;
    if (axis == 0) {
        s = mk(-h.x, hi ? h.y : -h.y, lo ? h.z : -h.z); e = mk(h.x, s.y, s.z);
        sId = (hi ? 2 : 0) + (lo ? 1 : 0); eId = sId + 4;
    } else if (axis == 1) {
        s = mk(hi ? h.x : -h.x, -h.y, lo ? h.z : -h.z); e = mk(s.x, h.y, s.z);
        sId = (hi ? 4 : 0) + (lo ? 1 : 0); eId = sId + 2;
    } else {
        s = mk(hi ? h.x : -h.x, lo ? h.y : -h.y, -h.z); e = mk(s.x, s.y, h.z);
        sId = (hi ? 4 : 0) + (lo ? 2 : 0); eId = sId + 1;
    }
}

// The two box edges along the local axis the mtd is perpendicular to, furthest
// along it (FindHighestIndices: first strict maximum, then the first strict
// maximum of the rest).
__device__ __forceinline__ void FurthestEdges(V3 h, V3 m, V3 s[2], V3 e[2], int sId[2], int eId[2]) {
    int axis;
    float p, pv, q, qv;
    if (fabsf(m.x) < kEps) { axis = 0; p = h.y; pv = m.y; q = h.z; qv = m.z; }
    else if (fabsf(m.y) < kEps) { axis = 1; p = h.x; pv = m.x; q = h.z; qv = m.z; }
    else { axis = 2; p = h.x; pv = m.x; q = h.y; qv = m.y; }
    float dots[4] = {-p * pv - q * qv, -p * pv + q * qv, p * pv - q * qv, p * pv + q * qv};
    int hi = 0;
    float hv = dots[0];
    for (int i = 1; i < 4; i++)
        if (dots[i] > hv) { hi = i; hv = dots[i]; }
    int second = 0;
    float sv = -3.402823466e+38f;
    for (int i = 0; i < 4; i++)
        if (i != hi && dots[i] > sv) { second = i; sv = dots[i]; }
    EdgeData(hi, axis, h, s[0], e[0], sId[0], eId[0]);
    EdgeData(second, axis, h, s[1], e[1], sId[1], eId[1]);
}

// BoxBoxCollider.GetClosestPointsBetweenSegments (:2918-2990).
__device__ __forceinline__ bool SegmentClosest(V3 p1, V3 q1, V3 p2, V3 q2, V3& c1, V3& c2) {
    V3 d1 = q1 - p1, d2 = q2 - p2, r = p1 - p2;
    float a = len2(d1), e = len2(d2), f = dot(d2, r);
    float s, t;
    if (a <= kEps && e <= kEps) return false;
    if (a <= kEps) {
        s = 0.0f;
        t = f / e;
        if (t < 0 || t > 1) return false;
    } else {
        float c = dot(d1, r);
        if (e <= kEps) {
            t = 0.0f;
            s = clampf(-c / a, 0.0f, 1.0f);
        } else {
            float b = dot(d1, d2);
            float denom = a * e - b * b;
            if (denom != 0.0f) {
                s = (b * f - c * e) / denom;
                if (s < 0 || s > 1) return false;
            } else {
                s = .5f;
            }
            t = (b * s + f) / e;
            if (t < 0 || t > 1) return false;
        }
    }
    c1 = scale(d1, s) + p1;
    c2 = scale(d2, t) + p2;
    return true;
}

__device__ __forceinline__ void EdgeEdge(V3 ha, V3 hb, V3 pa, const V3 oa[3], V3 pb, const V3 ob[3], V3 mtd, Cands& out) {
    V3 mA = TimesRows(-mtd, oa), mB = TimesRows(mtd, ob);
    V3 sa[2], ea[2], sb[2], eb[2];
    int saId[2], eaId[2], sbId[2], ebId[2];
    FurthestEdges(ha, mA, sa, ea, saId, eaId);
    FurthestEdges(hb, mB, sb, eb, sbId, ebId);
    for (int k = 0; k < 2; k++) {
        sa[k] = RowTimes(sa[k], oa) + pa; ea[k] = RowTimes(ea[k], oa) + pa;
        sb[k] = RowTimes(sb[k], ob) + pb; eb[k] = RowTimes(eb[k], ob) + pb;
    }
    out.n = 0;
    for (int k = 0; k < 4; k++) {
        const int i = k >> 1, j = k & 1;
        V3 onA, onB;
        if (SegmentClosest(sa[i], ea[i], sb[j], eb[j], onA, onB)) {
            float d = dot(onA - onB, mtd);
            if (d < 0) out.add(onA, d, EdgeId(saId[i], eaId[i]) * 2549 + EdgeId(sbId[j], ebId[j]) * 2857);
        }
    }
}

struct Face {
    V3 v[4], normal;
    float width, height;
    int id[4];
};

// GetNearestFace: the face whose normal is most aligned with `m` (none when
// no component strictly dominates, as in the reference).
__device__ __forceinline__ void NearestFace(V3 pos, const V3 o[3], V3 m, V3 h, Face& f) {
    float dd[3] = {dot(o[0], m), dot(o[1], m), dot(o[2], m)};
    float ad[3] = {fabsf(dd[0]), fabsf(dd[1]), fabsf(dd[2])};
    int k = -1;
    if (ad[0] > ad[1] && ad[0] > ad[2]) k = 0;
    else if (ad[1] > ad[0] && ad[1] > ad[2]) k = 1;
    else if (ad[2] > ad[0] && ad[2] > ad[1]) k = 2;
    for (int i = 0; i < 4; i++) { f.v[i] = mk(0, 0, 0); f.id[i] = 0; }
    f.normal = mk(0, 0, 0);
    f.width = f.height = 0;
    if (k < 0) return;
    const bool neg = dd[k] < 0;
    float hw = h.x, hh = h.y, hl = h.z;
    int bit;
    // corner signs (x, y, z) of V1..V4 on each face family, from :6076-6170
    int sx[4], sy[4], sz[4];
    if (k == 0) {
        if (neg) { hw = -hw; bit = 0; } else bit = 1;
        const int X[4] = {1, 1, 1, 1}, Y[4] = {1, -1, -1, 1}, Z[4] = {1, 1, -1, -1};
        for (int i = 0; i < 4; i++) { sx[i] = X[i]; sy[i] = Y[i]; sz[i] = Z[i]; }
        f.width = hh * 2; f.height = hl * 2;
        f.id[0] = bit + 2 + 4; f.id[1] = bit + 4; f.id[2] = bit + 2; f.id[3] = bit;
    } else if (k == 1) {
        if (neg) { hh = -hh; bit = 0; } else bit = 2;
        const int X[4] = {1, -1, -1, 1}, Y[4] = {1, 1, 1, 1}, Z[4] = {1, 1, -1, -1};
        for (int i = 0; i < 4; i++) { sx[i] = X[i]; sy[i] = Y[i]; sz[i] = Z[i]; }
        f.width = hw * 2; f.height = hl * 2;
        f.id[0] = 1 + bit + 4; f.id[1] = bit + 4; f.id[2] = 1 + bit; f.id[3] = bit;
    } else {
        if (neg) { hl = -hl; bit = 0; } else bit = 4;
        const int X[4] = {1, -1, -1, 1}, Y[4] = {1, 1, -1, -1}, Z[4] = {1, 1, 1, 1};
        for (int i = 0; i < 4; i++) { sx[i] = X[i]; sy[i] = Y[i]; sz[i] = Z[i]; }
        f.width = hw * 2; f.height = hh * 2;
        f.id[0] = 1 + 2 + bit; f.id[1] = 2 + bit; f.id[2] = 1 + bit; f.id[3] = bit;
    }
    for (int i = 0; i < 4; i++) {
        float x = sx[i] > 0 ? hw : -hw, y = sy[i] > 0 ? hh : -hh, z = sz[i] > 0 ? hl : -hl;
        // Matrix.Transform by the orientation rows and the position (Matrix.cs:717-725)
        f.v[i] = mk(x * o[0].x + y * o[1].x + z * o[2].x + pos.x, x * o[0].y + y * o[1].y + z * o[2].y + pos.y,
                    x * o[0].z + y * o[1].z + z * o[2].z + pos.z);
    }
    f.normal = neg ? -o[k] : o[k];
}

struct ClipEdge {
    V3 a, b, perp;
    int id;
};
// BoxFace.GetEdge (:6223-6270): edge i runs V[i] -> V[i+1]; its normal in the
// face plane points away from V[i+2].
__device__ __forceinline__ ClipEdge EdgeOf(const Face& f, int i) {
    ClipEdge c;
    const int ib = (i + 1) & 3, in = (i + 2) & 3;
    c.a = f.v[i];
    c.b = f.v[ib];
    c.id = EdgeId(f.id[i], f.id[ib]);
    V3 dir = c.b - c.a;
    float inverse = dr::InvSqrtAsDouble(dir.x * dir.x + dir.y * dir.y + dir.z * dir.z);
    dir = mk(dir.x * inverse, dir.y * inverse, dir.z * inverse);
    c.perp = cross(dir, f.normal);
    if (dot(c.perp, f.v[in] - c.a) > 0) c.perp = -c.perp;
    return c;
}

// ComputeIntersection (:6007-6040).
__device__ __forceinline__ bool Intersect(V3 a1, V3 a2, const ClipEdge& ce, V3& at) {
    V3 dir = a2 - a1;
    float t = dot(ce.a - a1, ce.perp) / dot(dir, ce.perp);
    if (t < 0 || t > 1) return false;
    at = scale(dir, t) + a1;
    V3 along = ce.b - ce.a;
    t = dot(along, at - ce.a);
    return !(t < 0 || t > len2(along));
}

// ClipFacesDirect (:4517-5278): inside flags per vertex as bits
// 1 = MaxX, 2 = MinX, 4 = MaxY, 8 = MinY.
__device__ __forceinline__ void ClipFaces(const Face& clip, const Face& face, V3 mtd, Cands& out) {
    V3 clipX = clip.v[3] - clip.v[2], clipY = clip.v[1] - clip.v[2];
    float icw = 1 / clip.width, ich = 1 / clip.height;
    float icw2 = icw * icw;
    clipX = mk(clipX.x * icw2, clipX.y * icw2, clipX.z * icw2);
    float ich2 = ich * ich;
    clipY = mk(clipY.x * ich2, clipY.y * ich2, clipY.z * ich2);
    V3 faceX = face.v[3] - face.v[2], faceY = face.v[1] - face.v[2];
    float ifw = 1 / face.width, ifh = 1 / face.height;
    float ifw2 = ifw * ifw;
    faceX = mk(faceX.x * ifw2, faceX.y * ifw2, faceX.z * ifw2);
    float ifh2 = ifh * ifh;
    faceY = mk(faceY.x * ifh2, faceY.y * ifh2, faceY.z * ifh2);
    V3 cc = clip.v[0] + clip.v[2];
    float ccx = dot(cc, clipX), ccy = dot(cc, clipY);
    ccx *= .5f;
    ccy *= .5f;
    V3 fc = face.v[0] + face.v[2];
    float fcx = dot(fc, faceX), fcy = dot(fc, faceY);
    fcx *= .5f;
    fcy *= .5f;
    float ex = .5f + .01f * icw, ey = .5f + .01f * ich;
    const float cMaxX = ccx + ex, cMaxY = ccy + ey, cMinX = ccx - ex, cMinY = ccy - ey;
    ex = .5f + .01f * ifw;
    ey = .5f + .01f * ifh;
    const float fMaxX = fcx + ex, fMaxY = fcy + ey, fMinX = fcx - ex, fMinY = fcy - ey;
    int fv[4], cv[4];
    for (int v = 0; v < 4; v++) {
        float dx = dot(clipX, face.v[v]), dy = dot(clipY, face.v[v]);
        fv[v] = (dx < cMaxX ? 1 : 0) | (dx > cMinX ? 2 : 0) | (dy < cMaxY ? 4 : 0) | (dy > cMinY ? 8 : 0);
        dx = dot(faceX, clip.v[v]);
        dy = dot(faceY, clip.v[v]);
        cv[v] = (dx < fMaxX ? 1 : 0) | (dx > fMinX ? 2 : 0) | (dy < fMaxY ? 4 : 0) | (dy > fMinY ? 8 : 0);
    }
    const float clipDot = dot(clip.v[0], mtd);
    out.n = 0;
    // face vertices inside the clip face, kept at non-positive depth
    for (int v = 0; v < 4; v++)
        if (fv[v] == 15) {
            float depth = dot(face.v[v], mtd) - clipDot;
            if (depth <= 0) out.add(face.v[v], depth, face.id[v]);
        }
    if (out.n >= 4) return;
    // clip vertices inside the face, projected onto its plane
    const float b = dot(face.v[0], face.normal);
    for (int v = 0; v < 4; v++)
        if (cv[v] == 15) {
            float a = dot(clip.v[v], face.normal);
            V3 p = clip.v[v] - scale(face.normal, a - b);
            float depth = dot(p, mtd) - clipDot;
            if (depth <= 0) out.add(p, depth, clip.id[v] + 8);
        }
    if (out.n >= 4) return;
    // Face edges crossing the clip edges v1v2 (MaxY), v2v3 (MinX), v3v4
    // (MinY), v4v1 (MaxX).  A vertex outside a clip edge tries its lower
    // neighbour then its higher one (v1: v2, v4) -- on edge v3v4, v4 tries v3
    // before v1.  Candidates past eight are dropped; depths are taken once at
    // the end.
    const int flagOf[4] = {4, 2, 8, 1};
    const int first = out.n;
    for (int e = 0; e < 4; e++) {
        const ClipEdge ce = EdgeOf(clip, e);
        const int fl = flagOf[e];
        for (int v = 0; v < 4; v++) {
            if (fv[v] & fl) continue;
            int n0 = (v + 1) & 3, n1 = (v + 3) & 3;
            int lo = n0 < n1 ? n0 : n1, hi = n0 < n1 ? n1 : n0;
            if (e == 2 && v == 3) { int t = lo; lo = hi; hi = t; }
            for (int w = 0; w < 2; w++) {
                const int n = w == 0 ? lo : hi;
                if (!(fv[n] & fl)) continue;
                // the face edge between v and n, in the reference's argument order
                const bool wrap = (v == 0 && n == 3) || (v == 3 && n == 0);
                const int p = wrap ? 3 : (v < n ? v : n), q = (p + 1) & 3;
                V3 at;
                if (out.n < 8 && Intersect(face.v[p], face.v[q], ce, at))
                    out.add(at, 0.f, EdgeId(face.id[p], face.id[q]) * 2549 + ce.id * 2857);
            }
        }
    }
    // depths of the edge candidates; positive ones dropped, order kept
    int kept = first;
    for (int i = first; i < out.n; i++) {
        float depth = dot(out.p[i], mtd) - clipDot;
        if (depth <= 0) {
            out.p[kept] = out.p[i];
            out.d[kept] = depth;
            out.id[kept] = out.id[i];
            kept++;
        }
    }
    out.n = kept;
}

// PruneContactsMaxDistance (:3612-3700): deepest, furthest from it, and the
// extremes along mtd x (furthest - deepest).
__device__ __forceinline__ void Prune(V3 mtd, Cands& c) {
    int deep = 0;
    for (int i = 1; i < c.n; i++)
        if (c.d[i] > c.d[deep]) deep = i;
    int far = 0;
    float farDist = len2(c.p[deep] - c.p[0]);
    for (int i = 1; i < c.n; i++) {
        float dd = len2(c.p[deep] - c.p[i]);
        if (dd > farDist) { farDist = dd; far = i; }
    }
    V3 yAxis = cross(mtd, c.p[far] - c.p[deep]);
    int mn = 0, mx = 0;
    float minY = dot(c.p[0], yAxis), maxY = minY;
    for (int i = 1; i < c.n; i++) {
        float d = dot(yAxis, c.p[i]);
        if (d < minY) { minY = d; mn = i; }
        else if (d > maxY) { maxY = d; mx = i; }
    }
    const int pick[4] = {deep, far, mn, mx};
    V3 p[4];
    float d[4];
    int id[4];
    for (int k = 0; k < 4; k++) { p[k] = c.p[pick[k]]; d[k] = c.d[pick[k]]; id[k] = c.id[pick[k]]; }
    for (int k = 0; k < 4; k++) { c.p[k] = p[k]; c.d[k] = d[k]; c.id[k] = id[k]; }
    c.n = 4;
}

// AreBoxesColliding (:1494-2388).  Returns false when an axis separates the
// boxes; otherwise the contacts and the minimum axis (pointing from B to A).
__device__ __forceinline__ bool BoxBox(V3 ha, V3 hb, V3 pa, float4 qa, V3 pb, float4 qb, V3& axis, Cands& out) {
    V3 A[3], B[3];
    Rows(qa, A);
    Rows(qb, B);
    const float av[3] = {ha.x, ha.y, ha.z}, bv[3] = {hb.x, hb.y, hb.z};
    V3 t0 = pb - pa;
    float R[3][3], AR[3][3], t[3];
    float minD = -3.402823466e+38f;
    V3 minAxis = mk(0, 0, 0);
    int feature = 2;
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 3; j++) {
            R[i][j] = A[i].x * B[j].x + A[i].y * B[j].y + A[i].z * B[j].z;
            AR[i][j] = fabsf(R[i][j]) + kEps;
        }
        t[i] = t0.x * A[i].x + t0.y * A[i].y + t0.z * A[i].z;
        const float rarb = av[i] + bv[0] * AR[i][0] + bv[1] * AR[i][1] + bv[2] * AR[i][2];
        if (t[i] > rarb || t[i] < -rarb) return false;
        const float d = t[i] > 0 ? t[i] - rarb : -t[i] - rarb;
        if (d > minD) { minD = d; minAxis = t[i] > 0 ? -A[i] : A[i]; feature = 0; }
    }
    minD += .01f;  // antiBBias
    for (int j = 0; j < 3; j++) {
        const float rarb = bv[j] + av[0] * AR[0][j] + av[1] * AR[1][j] + av[2] * AR[2][j];
        const float tl = t[0] * R[0][j] + t[1] * R[1][j] + t[2] * R[2][j];
        if (tl > rarb || tl < -rarb) return false;
        const float d = tl > 0 ? tl - rarb : -tl - rarb;
        if (d > minD) { minD = d; minAxis = tl > 0 ? -B[j] : B[j]; feature = 1; }
    }
    if (feature != 1) minD -= .01f;
    minD += .01f;  // antiEdgeBias
    for (int i = 0; i < 3; i++) {
        const int i1 = i == 0 ? 1 : 0, i2 = i == 2 ? 1 : 2;
        const int c1 = i == 2 ? 0 : i + 1, c2 = i == 0 ? 2 : i - 1;
        for (int j = 0; j < 3; j++) {
            const int j1 = j == 0 ? 1 : 0, j2 = j == 2 ? 1 : 2;
            const float rarb = av[i1] * AR[i2][j] + av[i2] * AR[i1][j] + bv[j1] * AR[i][j2] + bv[j2] * AR[i][j1];
            const float tl = t[c2] * R[c1][j] - t[c1] * R[c2][j];
            // the parallel test reads absBR[j][i], the reference's index order
            if (AR[j][i] < 1 && (tl > rarb || tl < -rarb)) return false;
            const V3 ai = A[i], bj = B[j];
            V3 ta = tl > 0 ? mk(bj.y * ai.z - bj.z * ai.y, bj.z * ai.x - bj.x * ai.z, bj.x * ai.y - bj.y * ai.x)
                           : mk(ai.y * bj.z - ai.z * bj.y, ai.z * bj.x - ai.x * bj.z, ai.x * bj.y - ai.y * bj.x);
            const float inv = 1 / __fsqrt_rn(len2(ta));
            const float d = (tl > 0 ? tl - rarb : -tl - rarb) * inv;
            if (d > minD) {
                feature = 2;
                minD = d;
                minAxis = mk(ta.x * inv, ta.y * inv, ta.z * inv);
            }
        }
    }
    axis = minAxis;
    if (feature == 2) {
        EdgeEdge(ha, hb, pa, A, pb, B, minAxis, out);
    } else {
        Face fa, fb;
        NearestFace(pa, A, -minAxis, ha, fa);
        NearestFace(pb, B, minAxis, hb, fb);
        if (feature == 0) ClipFaces(fa, fb, -minAxis, out);
        else ClipFaces(fb, fa, minAxis, out);
        if (out.n > 4) Prune(minAxis, out);
    }
    return true;
}

// One-contact testers' output (ContactData).
struct One {
    V3 p, n;
    float depth;
};

// SphereTester.AreSpheresColliding.
__device__ __forceinline__ bool SphereSphere(float ra, float rb, V3 pa, V3 pb, float maxDist, One& c) {
    const float rs = ra + rb;
    V3 d = pb - pa;
    float dist = len2(d);
    const float lim = rs + maxDist;
    if (!(dist < lim * lim)) return false;
    c.p = rs > kEps ? scale(d, ra / rs) : mk(0, 0, 0);
    c.p = c.p + pa;
    dist = __fsqrt_rn(dist);
    if (dist > kBigEps) {
        float inv = 1 / dist;  // Vector3.Divide
        c.n = scale(d, inv);
    } else {
        c.n = mk(0, 1, 0);
    }
    c.depth = rs - dist;
    return true;
}

// BoxSphereTester.AreShapesColliding (box is body A, sphere body B).
__device__ __forceinline__ bool BoxSphere(V3 h, float r, V3 pa, float4 qa, V3 pb, float maxDist, One& c) {
    float4 conj = make_float4(-qa.x, -qa.y, -qa.z, qa.w);
    V3 local = QRot(pb - pa, conj);
    V3 lc = mk(clampf(local.x, -h.x, h.x), clampf(local.y, -h.y, h.y), clampf(local.z, -h.z, h.z));
    c.p = QRot(lc, qa) + pa;
    V3 off = pb - c.p;
    float l = len2(off);
    const float lim = r + maxDist;
    if (l > lim * lim) return false;
    if (l > kEps) {
        l = __fsqrt_rn(l);
        float inv = 1 / l;
        c.n = scale(off, inv);
        c.depth = r - l;
    } else {
        V3 pd = mk(lc.x < 0 ? lc.x + h.x : h.x - lc.x, lc.y < 0 ? lc.y + h.y : h.y - lc.y,
                   lc.z < 0 ? lc.z + h.z : h.z - lc.z);
        if (pd.x < pd.y && pd.x < pd.z) { c.n = mk(lc.x > 0 ? 1.f : -1.f, 0, 0); c.depth = pd.x; }
        else if (pd.y < pd.z) { c.n = mk(0, lc.y > 0 ? 1.f : -1.f, 0); c.depth = pd.y; }
        else { c.n = mk(0, 0, lc.z > 0 ? 1.f : -1.f); c.depth = pd.z; }
        c.depth += r;
        c.n = QRot(c.n, qa);
    }
    return true;
}

// The manifold's contacts in solver order (the constraint's penetration
// list) plus the manifold's own list order.
struct Kept {
    float4 cp[4], cn[4], oa[4], ob[4];
    float4 cf[4];  // NONCONVEX: each contact's friction direction and impulse
    float acc[4];
    int n;
    int list[4];  // list position -> solver index
};

// ContactManifold.Remove of list entry i: the list moves its last entry into
// the gap (RawList.FastRemoveAt); the constraint removes its penetration child
// (and, NONCONVEX, the contact's friction child) keeping order (RawList.RemoveAt).
__device__ __forceinline__ void RemoveListAt(Kept& k, int i) {
    const int p = k.list[i];
    k.list[i] = k.list[k.n - 1];
    for (int q = p; q + 1 < k.n; q++) {
        k.cp[q] = k.cp[q + 1]; k.cn[q] = k.cn[q + 1]; k.oa[q] = k.oa[q + 1]; k.ob[q] = k.ob[q + 1];
        k.cf[q] = k.cf[q + 1];
        k.acc[q] = k.acc[q + 1];
    }
    k.n--;
    for (int q = 0; q < k.n; q++)
        if (k.list[q] > p) k.list[q]--;
}

// ContactManifold.Add: appended to both lists with a fresh (zero) impulse.
__device__ __forceinline__ void AddContact(Kept& k, V3 p, V3 n, float depth, int id) {
    const int s = k.n;
    k.cp[s] = make_float4(p.x, p.y, p.z, depth);
    k.cn[s] = make_float4(n.x, n.y, n.z, __int_as_float(id));
    k.oa[s] = make_float4(0, 0, 0, 0);
    k.ob[s] = make_float4(0, 0, 0, 0);
    k.cf[s] = make_float4(0, 0, 0, 0);  // ContactFrictionConstraint.Setup: linearA = 0, impulse 0
    k.acc[s] = 0.f;
    k.list[s] = s;
    k.n++;
}

// The narrow phase of one GENERATED manifold slot.
__device__ __forceinline__ void CollideManifold(const ManifoldSoA& m, const BodySoA& b, const float4* __restrict__ shape,
                                                int s, const StepParams& prm) {
    int4 h = m.head[s];
    const int cap = m.capacity;
    const int ia = h.x, ib = h.y;
    const float4 sa = shape[ia], sb = shape[ib];
    const float4 pa4 = b.pos[ia], pb4 = b.pos[ib], qa = b.quat[ia], qb = b.quat[ib];
    const V3 pa = mk(pa4.x, pa4.y, pa4.z), pb = mk(pb4.x, pb4.y, pb4.z);
    const int ta = __float_as_int(sa.w), tb = __float_as_int(sb.w);
    Kept k;
    k.n = h.z & 0xff;
    float4 fr = m.fricacc[s];
    const uint32_t code = (uint32_t)__float_as_int(fr.w) ^ 0xE4u;
    const float4 pen = m.penacc[s];
    const float accs[4] = {pen.x, pen.y, pen.z, pen.w};
    const bool nonConvex = ((uint32_t)h.z >> 8) & kManifoldNonConvex;
    for (int q = 0; q < 4; q++) {
        if (q < k.n) {
            k.cp[q] = m.cpos[q * cap + s];
            k.cn[q] = m.cnrm[q * cap + s];
            k.oa[q] = m.offA[q * cap + s];
            k.ob[q] = m.offB[q * cap + s];
            k.cf[q] = nonConvex ? m.cfr[q * cap + s] : make_float4(0, 0, 0, 0);
            k.acc[q] = accs[q];
            k.list[q] = (int)((code >> (2 * q)) & 3u);
        }
    }
    const int before = k.n;
    bool setup = false;  // the first contact after none: friction is set up again
    if (ta == 1 && tb == 1) {
        V3 axis;
        Cands c;
        c.n = 0;
        if (BoxBox(mk(sa.x, sa.y, sa.z), mk(sb.x, sb.y, sb.z), pa, qa, pb, qb, axis, c)) {
            axis = -axis;
            int toRemove[4], nr = 0;
            for (int i = 0; i < k.n; i++) {
                const int pi = k.list[i];
                const int id = __float_as_int(k.cn[pi].w);
                bool found = false;
                for (int j = c.n - 1; j >= 0; j--) {
                    if (c.id[j] == id) {
                        found = true;
                        k.cp[pi] = make_float4(c.p[j].x, c.p[j].y, c.p[j].z, -c.d[j]);
                        k.cn[pi] = make_float4(axis.x, axis.y, axis.z, k.cn[pi].w);
                        c.removeAt(j);
                        break;
                    }
                }
                if (!found) toRemove[nr++] = i;
            }
            for (int r = nr - 1; r >= 0; r--) RemoveListAt(k, toRemove[r]);
            const bool emptied = before > 0 && k.n == 0;
            for (int j = 0; j < c.n; j++) {
                if (k.n == 0) setup = true;
                AddContact(k, c.p[j], axis, -c.d[j], c.id[j]);
            }
            if (emptied) fr = make_float4(0.f, 0.f, 0.f, fr.w);
        } else {
            for (int i = k.n - 1; i >= 0; i--) RemoveListAt(k, i);
            if (before > 0) fr = make_float4(0.f, 0.f, 0.f, fr.w);
        }
    } else {
        One c;
        const bool hit = ta == 2 ? SphereSphere(sa.x, sb.x, pa, pb, prm.maximumContactDistance, c)
                                 : BoxSphere(mk(sa.x, sa.y, sa.z), sb.x, pa, qa, pb, prm.maximumContactDistance, c);
        const bool previously = k.n > 0;
        if (hit) {
            if (!previously && c.depth >= 0) {
                setup = true;
                AddContact(k, c.p, c.n, c.depth, 0);
            } else if (previously) {
                const int p = 0;
                k.cp[p] = make_float4(c.p.x, c.p.y, c.p.z, c.depth);
                k.cn[p] = make_float4(c.n.x, c.n.y, c.n.z, k.cn[p].w);
            }
        } else if (previously) {
            RemoveListAt(k, 0);
            fr = make_float4(0.f, 0.f, 0.f, fr.w);
        }
    }
    // write back: contacts in solver order, the list order, impulses
    uint32_t out = 0;
    for (int q = 0; q < 4; q++) out |= (uint32_t)(q < k.n ? k.list[q] : q) << (2 * q);
    fr.w = __int_as_float((int)(out ^ 0xE4u));
    for (int q = 0; q < 4; q++) {
        if (q < k.n) {
            m.cpos[q * cap + s] = k.cp[q];
            m.cnrm[q * cap + s] = k.cn[q];
            m.offA[q * cap + s] = k.oa[q];
            m.offB[q * cap + s] = k.ob[q];
        }
        if (nonConvex && q < (k.n > before ? k.n : before))
            m.cfr[q * cap + s] = q < k.n ? k.cf[q] : make_float4(0, 0, 0, 0);
    }
    m.penacc[s] = make_float4(k.n > 0 ? k.acc[0] : 0.f, k.n > 1 ? k.acc[1] : 0.f, k.n > 2 ? k.acc[2] : 0.f,
                              k.n > 3 ? k.acc[3] : 0.f);
    m.fricacc[s] = fr;
    if (setup) {
        float4 ax = m.saxis[s];
        m.saxis[s] = make_float4(0.f, 0.f, 0.f, ax.w);  // SlidingFrictionTwoAxis.Setup: linearA = 0
    }
    if (k.n != before) {
        h.z = (h.z & ~0xff) | k.n;
        m.head[s] = h;
    }
}

}  // namespace nphase
}  // namespace bepugpu
