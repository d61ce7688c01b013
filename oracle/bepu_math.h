// Oracle math -- test infrastructure only.
//
// Restates, operation for operation, the BEPUutilities arithmetic the solver
// path uses, so that float rounding follows the reference's evaluation order.
// Compile with -ffp-contract=off: C# never fuses a*b+c.  Where the reference
// calls System.Math (double) the restatement does the same in double.
#pragma once
#include <cmath>

namespace oracle {

struct Vec3 { float X = 0, Y = 0, Z = 0; };
struct Quat { float X = 0, Y = 0, Z = 0, W = 1; };
struct Mat3 {
    float M11 = 0, M12 = 0, M13 = 0;
    float M21 = 0, M22 = 0, M23 = 0;
    float M31 = 0, M32 = 0, M33 = 0;
};
struct Mat2 { float M11 = 0, M12 = 0, M21 = 0, M22 = 0; };
struct Mat2x3 { float M11 = 0, M12 = 0, M13 = 0, M21 = 0, M22 = 0, M23 = 0; };
struct Mat3x2 { float M11 = 0, M12 = 0, M21 = 0, M22 = 0, M31 = 0, M32 = 0; };

// MathHelper.Max/Min/Clamp (BEPUutilities/MathHelper.cs:58-88)
inline float Max(float a, float b) { return a > b ? a : b; }
inline float Min(float a, float b) { return a < b ? a : b; }
inline float Clamp(float v, float lo, float hi) {
    if (v < lo) return lo;
    else if (v > hi) return hi;
    return v;
}

// Toolbox constants (BEPUutilities/Toolbox.cs:20,25)
constexpr float Epsilon = 1e-7f;
constexpr float BigEpsilon = 1e-5f;

// Vector3 (BEPUutilities/Vector3.cs)
inline Vec3 Add(const Vec3& a, const Vec3& b) { return {a.X + b.X, a.Y + b.Y, a.Z + b.Z}; }
inline Vec3 Subtract(const Vec3& a, const Vec3& b) { return {a.X - b.X, a.Y - b.Y, a.Z - b.Z}; }
inline Vec3 Multiply(const Vec3& a, float s) { return {a.X * s, a.Y * s, a.Z * s}; }
inline float Dot(const Vec3& a, const Vec3& b) { return a.X * b.X + a.Y * b.Y + a.Z * b.Z; }
inline float LengthSquared(const Vec3& a) { return a.X * a.X + a.Y * a.Y + a.Z * a.Z; }
// Vector3.Length (Vector3.cs:73-76)
inline float Length(const Vec3& a) { return (float)std::sqrt((double)(a.X * a.X + a.Y * a.Y + a.Z * a.Z)); }
// Vector3.Cross
inline Vec3 Cross(const Vec3& a, const Vec3& b) {
    return {a.Y * b.Z - a.Z * b.Y, a.Z * b.X - a.X * b.Z, a.X * b.Y - a.Y * b.X};
}
// Vector3.Normalize (Vector3.cs:81-87)
inline void Normalize(Vec3& v) {
    float inverse = (float)(1.0 / std::sqrt((double)(v.X * v.X + v.Y * v.Y + v.Z * v.Z)));
    v.X *= inverse; v.Y *= inverse; v.Z *= inverse;
}

// Quaternion (BEPUutilities/Quaternion.cs:51-79, 262-269, 509-535)
inline Quat QAdd(const Quat& a, const Quat& b) { return {a.X + b.X, a.Y + b.Y, a.Z + b.Z, a.W + b.W}; }
inline Quat QMultiply(const Quat& a, const Quat& b) {
    float x = a.X, y = a.Y, z = a.Z, w = a.W;
    float bX = b.X, bY = b.Y, bZ = b.Z, bW = b.W;
    Quat r;
    r.X = x * bW + bX * w + y * bZ - z * bY;
    r.Y = y * bW + bY * w + z * bX - x * bZ;
    r.Z = z * bW + bZ * w + x * bY - y * bX;
    r.W = w * bW - x * bX - y * bY - z * bZ;
    return r;
}
inline void QNormalize(Quat& q) {
    float inverse = (float)(1.0 / std::sqrt((double)(q.X * q.X + q.Y * q.Y + q.Z * q.Z + q.W * q.W)));
    q.X *= inverse; q.Y *= inverse; q.Z *= inverse; q.W *= inverse;
}
inline Vec3 QTransform(const Vec3& v, const Quat& r) {
    float x2 = r.X + r.X, y2 = r.Y + r.Y, z2 = r.Z + r.Z;
    float xx2 = r.X * x2, xy2 = r.X * y2, xz2 = r.X * z2;
    float yy2 = r.Y * y2, yz2 = r.Y * z2, zz2 = r.Z * z2;
    float wx2 = r.W * x2, wy2 = r.W * y2, wz2 = r.W * z2;
    Vec3 o;
    o.X = v.X * (1.f - yy2 - zz2) + v.Y * (xy2 - wz2) + v.Z * (xz2 + wy2);
    o.Y = v.X * (xy2 + wz2) + v.Y * (1.f - xx2 - zz2) + v.Z * (yz2 - wx2);
    o.Z = v.X * (xz2 - wy2) + v.Y * (yz2 + wx2) + v.Z * (1.f - xx2 - yy2);
    return o;
}

// Matrix3x3 (BEPUutilities/Matrix3x3.cs)
inline Mat3 CreateFromQuaternion(const Quat& q) {  // :1303-1328
    float qX2 = q.X + q.X, qY2 = q.Y + q.Y, qZ2 = q.Z + q.Z;
    float XX = qX2 * q.X, YY = qY2 * q.Y, ZZ = qZ2 * q.Z;
    float XY = qX2 * q.Y, XZ = qX2 * q.Z, XW = qX2 * q.W;
    float YZ = qY2 * q.Z, YW = qY2 * q.W, ZW = qZ2 * q.W;
    Mat3 r;
    r.M11 = 1 - YY - ZZ; r.M21 = XY - ZW; r.M31 = XZ + YW;
    r.M12 = XY + ZW; r.M22 = 1 - XX - ZZ; r.M32 = YZ - XW;
    r.M13 = XZ - YW; r.M23 = YZ + XW; r.M33 = 1 - XX - YY;
    return r;
}
inline Mat3 Multiply(const Mat3& a, const Mat3& b) {  // :766-790
    Mat3 r;
    r.M11 = a.M11 * b.M11 + a.M12 * b.M21 + a.M13 * b.M31;
    r.M12 = a.M11 * b.M12 + a.M12 * b.M22 + a.M13 * b.M32;
    r.M13 = a.M11 * b.M13 + a.M12 * b.M23 + a.M13 * b.M33;
    r.M21 = a.M21 * b.M11 + a.M22 * b.M21 + a.M23 * b.M31;
    r.M22 = a.M21 * b.M12 + a.M22 * b.M22 + a.M23 * b.M32;
    r.M23 = a.M21 * b.M13 + a.M22 * b.M23 + a.M23 * b.M33;
    r.M31 = a.M31 * b.M11 + a.M32 * b.M21 + a.M33 * b.M31;
    r.M32 = a.M31 * b.M12 + a.M32 * b.M22 + a.M33 * b.M32;
    r.M33 = a.M31 * b.M13 + a.M32 * b.M23 + a.M33 * b.M33;
    return r;
}
inline Mat3 MultiplyTransposed(const Mat3& t, const Mat3& m) {  // :866-890 (t^T * m)
    Mat3 r;
    r.M11 = t.M11 * m.M11 + t.M21 * m.M21 + t.M31 * m.M31;
    r.M12 = t.M11 * m.M12 + t.M21 * m.M22 + t.M31 * m.M32;
    r.M13 = t.M11 * m.M13 + t.M21 * m.M23 + t.M31 * m.M33;
    r.M21 = t.M12 * m.M11 + t.M22 * m.M21 + t.M32 * m.M31;
    r.M22 = t.M12 * m.M12 + t.M22 * m.M22 + t.M32 * m.M32;
    r.M23 = t.M12 * m.M13 + t.M22 * m.M23 + t.M32 * m.M33;
    r.M31 = t.M13 * m.M11 + t.M23 * m.M21 + t.M33 * m.M31;
    r.M32 = t.M13 * m.M12 + t.M23 * m.M22 + t.M33 * m.M32;
    r.M33 = t.M13 * m.M13 + t.M23 * m.M23 + t.M33 * m.M33;
    return r;
}
inline Mat3 Subtract(const Mat3& a, const Mat3& b) {
    Mat3 r;
    r.M11 = a.M11 - b.M11; r.M12 = a.M12 - b.M12; r.M13 = a.M13 - b.M13;
    r.M21 = a.M21 - b.M21; r.M22 = a.M22 - b.M22; r.M23 = a.M23 - b.M23;
    r.M31 = a.M31 - b.M31; r.M32 = a.M32 - b.M32; r.M33 = a.M33 - b.M33;
    return r;
}
inline Mat3 CreateScale(float s) { Mat3 r; r.M11 = s; r.M22 = s; r.M33 = s; return r; }
inline Mat3 CreateCrossProduct(const Vec3& v) {  // :378-389
    Mat3 r;
    r.M11 = 0; r.M12 = -v.Z; r.M13 = v.Y;
    r.M21 = v.Z; r.M22 = 0; r.M23 = -v.X;
    r.M31 = -v.Y; r.M32 = v.X; r.M33 = 0;
    return r;
}
inline float Determinant(const Mat3& m) {  // :1231-1235
    return m.M11 * m.M22 * m.M33 + m.M12 * m.M23 * m.M31 + m.M13 * m.M21 * m.M32 -
           m.M31 * m.M22 * m.M13 - m.M32 * m.M23 * m.M11 - m.M33 * m.M21 * m.M12;
}
inline Mat3 Invert(const Mat3& m) {  // :505-534
    float d = 1 / Determinant(m);
    Mat3 r;
    r.M11 = (m.M22 * m.M33 - m.M23 * m.M32) * d;
    r.M12 = (m.M13 * m.M32 - m.M33 * m.M12) * d;
    r.M13 = (m.M12 * m.M23 - m.M22 * m.M13) * d;
    r.M21 = (m.M23 * m.M31 - m.M21 * m.M33) * d;
    r.M22 = (m.M11 * m.M33 - m.M13 * m.M31) * d;
    r.M23 = (m.M13 * m.M21 - m.M11 * m.M23) * d;
    r.M31 = (m.M21 * m.M32 - m.M22 * m.M31) * d;
    r.M32 = (m.M12 * m.M31 - m.M11 * m.M32) * d;
    r.M33 = (m.M11 * m.M22 - m.M12 * m.M21) * d;
    return r;
}
// Matrix3x3.Transform (:1071-1082): row vector times matrix
inline Vec3 Transform(const Vec3& v, const Mat3& m) {
    float vX = v.X, vY = v.Y, vZ = v.Z;
    return {vX * m.M11 + vY * m.M21 + vZ * m.M31,
            vX * m.M12 + vY * m.M22 + vZ * m.M32,
            vX * m.M13 + vY * m.M23 + vZ * m.M33};
}
// Matrix3x3.TransformTranspose (:1113-1123)
inline Vec3 TransformTranspose(const Vec3& v, const Mat3& m) {
    float vX = v.X, vY = v.Y, vZ = v.Z;
    return {vX * m.M11 + vY * m.M12 + vZ * m.M13,
            vX * m.M21 + vY * m.M22 + vZ * m.M23,
            vX * m.M31 + vY * m.M32 + vZ * m.M33};
}
// Matrix3x3.CreateFromAxisAngle (:1383-1400); sin/cos in double like System.Math
inline Mat3 CreateFromAxisAngle(const Vec3& axis, float angle) {
    float xx = axis.X * axis.X, yy = axis.Y * axis.Y, zz = axis.Z * axis.Z;
    float xy = axis.X * axis.Y, xz = axis.X * axis.Z, yz = axis.Y * axis.Z;
    float sinAngle = (float)std::sin((double)angle);
    float oneMinusCosAngle = 1 - (float)std::cos((double)angle);
    Mat3 r;
    r.M11 = 1 + oneMinusCosAngle * (xx - 1);
    r.M21 = -axis.Z * sinAngle + oneMinusCosAngle * xy;
    r.M31 = axis.Y * sinAngle + oneMinusCosAngle * xz;
    r.M12 = axis.Z * sinAngle + oneMinusCosAngle * xy;
    r.M22 = 1 + oneMinusCosAngle * (yy - 1);
    r.M32 = -axis.X * sinAngle + oneMinusCosAngle * yz;
    r.M13 = -axis.Y * sinAngle + oneMinusCosAngle * xz;
    r.M23 = axis.X * sinAngle + oneMinusCosAngle * yz;
    r.M33 = 1 + oneMinusCosAngle * (zz - 1);
    return r;
}

// Matrix2x2 (BEPUutilities/Matrix2x2.cs)
inline Mat2 Invert(const Mat2& m) {  // :160-174
    float d = 1 / (m.M11 * m.M22 - m.M12 * m.M21);
    Mat2 r;
    r.M11 = m.M22 * d;
    r.M12 = -m.M12 * d;
    r.M21 = -m.M21 * d;
    r.M22 = m.M11 * d;
    return r;
}
inline Mat2 Multiply(const Mat2x3& a, const Mat3x2& b) {  // :245-252
    Mat2 r;
    r.M11 = a.M11 * b.M11 + a.M12 * b.M21 + a.M13 * b.M31;
    r.M12 = a.M11 * b.M12 + a.M12 * b.M22 + a.M13 * b.M32;
    r.M21 = a.M21 * b.M11 + a.M22 * b.M21 + a.M23 * b.M31;
    r.M22 = a.M21 * b.M12 + a.M22 * b.M22 + a.M23 * b.M32;
    return r;
}
// Matrix2x3 (BEPUutilities/Matrix2x3.cs:94-111, 225-235)
inline Mat2x3 Multiply(const Mat2x3& a, const Mat3& b) {
    Mat2x3 r;
    r.M11 = a.M11 * b.M11 + a.M12 * b.M21 + a.M13 * b.M31;
    r.M12 = a.M11 * b.M12 + a.M12 * b.M22 + a.M13 * b.M32;
    r.M13 = a.M11 * b.M13 + a.M12 * b.M23 + a.M13 * b.M33;
    r.M21 = a.M21 * b.M11 + a.M22 * b.M21 + a.M23 * b.M31;
    r.M22 = a.M21 * b.M12 + a.M22 * b.M22 + a.M23 * b.M32;
    r.M23 = a.M21 * b.M13 + a.M22 * b.M23 + a.M23 * b.M33;
    return r;
}
inline Mat3x2 Transpose(const Mat2x3& m) {
    Mat3x2 r;
    r.M11 = m.M11; r.M12 = m.M21;
    r.M21 = m.M12; r.M22 = m.M22;
    r.M31 = m.M13; r.M32 = m.M23;
    return r;
}

}  // namespace oracle
