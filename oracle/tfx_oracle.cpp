// ============================================================================================
//  TressFX strand simulation + SDF collision -- THE ORACLE (test infrastructure only).
//
//  This file is a CPU restatement of the reference's compute shaders, kept in the reference's
//  operation order, templated on the arithmetic type (float = the FP32 transcription that the
//  CUDA path must match bit for bit; double = the FP64 drift reference).  It is a checker and
//  the timed CPU baseline; nothing in the shipped library links, loads or calls it.
//
//  Followed sources (paths inside the TressFX 4.1 project):
//    src/Shaders/TressFXSimulation.hlsl   : helpers :207-387, kernels :609-1001
//    src/Shaders/TressFXSDFCollision.hlsl : encoding :92-100, geometry :103-215,
//                                           kernels :301-412, lookup :414-527, collide :531-595
//    src/TressFX/TressFXSimulation.cpp:51-112    dispatch order, local-shape re-dispatch
//    src/TressFX/TressFXHairObject.cpp:380-437   constants that drive the kernels
//
//  Transcription rules (the CUDA kernels follow the same rules):
//    * every vector expression is evaluated component-wise, left to right, no FMA contraction
//      (built with -ffp-contract=off); division and sqrt are IEEE correctly rounded;
//    * dot(a,b) = a.x*b.x + a.y*b.y + a.z*b.z;  length(v) = sqrt(dot(v,v));
//      normalize(v) = v * (1 / length(v))   (the rsqrt-multiply form of HLSL's normalize,
//      with the reciprocal taken as an IEEE division);
//    * HLSL float literals are float constants here too (also in the FP64 variant);
//    * the damping decay exp(-damping*dt*60) is a per-dispatch uniform: it is evaluated once
//      per call with the C library's expf/exp and handed to every vertex (the CUDA side gets
//      the same host-evaluated value);
//    * float->int conversions saturate and map NaN to 0 (D3D ftoi semantics);
//    * min/max are IEEE minNum/maxNum (fmin/fmax), as D3D specifies them;
//    * the wind step of LengthConstriantsWindAndCollision reads sharedPos[i+nspg] while the
//      neighbour thread writes it, without a barrier (.hlsl:901-912).  On the wave64 hardware
//      the shader targets all lanes read before any lane writes; this restatement therefore
//      computes every wind displacement from the pre-wind positions (a Jacobi update).
//
//  Parity status: pinned bit for bit by tests/test_oracle_pin.py to the reference's own shader
//  source compiled as C++ (oracle/hlsl_ref), and carried to machines without the reference tree by
//  the golden fixtures under tests/golden.
// ============================================================================================

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace tfxo {

// ----------------------------------------------------------------------------- small vectors
template <class T> struct V3 { T x, y, z; };
template <class T> struct V4 { T x, y, z, w; };

template <class T> static inline V3<T> xyz(const V4<T>& a) { return {a.x, a.y, a.z}; }
template <class T> static inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> static inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> static inline V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> static inline V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> static inline V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> static inline V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> static inline V3<T> vdiv(V3<T> a, V3<T> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <class T> static inline T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> static inline V3<T> cross(V3<T> a, V3<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T> static inline T length(V3<T> a) { return std::sqrt(dot(a, a)); }
template <class T> static inline V3<T> normalize(V3<T> a) {
    T inv = T(1.0f) / std::sqrt(dot(a, a));
    return a * inv;
}
template <class T> static inline V3<T> vmin(V3<T> a, V3<T> b) { return {std::fmin(a.x, b.x), std::fmin(a.y, b.y), std::fmin(a.z, b.z)}; }
template <class T> static inline V3<T> vmax(V3<T> a, V3<T> b) { return {std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z)}; }

template <class T> static inline V4<T> ld4(const T* p, int64_t i) { const T* q = p + 4 * i; return {q[0], q[1], q[2], q[3]}; }
template <class T> static inline void st4(T* p, int64_t i, V4<T> v) { T* q = p + 4 * i; q[0] = v.x; q[1] = v.y; q[2] = v.z; q[3] = v.w; }
template <class T> static inline void st3(T* p, int64_t i, V3<T> v) { T* q = p + 4 * i; q[0] = v.x; q[1] = v.y; q[2] = v.z; }

// D3D ftoi: truncate toward zero, saturate, NaN -> 0.
template <class T> static inline int ftoi(T f) {
    if (!(f == f)) return 0;
    if (f >= T(2147483647.0)) return 2147483647;
    if (f <= T(-2147483648.0)) return (-2147483647 - 1);
    return (int)f;
}

// ----------------------------------------------------------------------------- constants block
// Byte layout of TressFXSimulationParams (src/TressFX/TressFXConstantBuffers.h:41-85,
// TRESSFX_COLLISION_CAPSULES = 0), which mirrors cbuffer tressfxSimParameters
// (TressFXSimulation.hlsl:49-79).
struct SimParamsF {
    float wind[4], wind1[4], wind2[4], wind3[4];
    float shape[4];        // damping, local stiffness, global stiffness, global range
    float gravTimeTip[4];  // gravity magnitude, time step, tip separation
    int32_t simInts[4];    // length iterations, local iterations, collision flag
    int32_t counts[4];     // strands per group, follow hairs per guide, verts per strand
    float vsp[4];          // VSP coefficient, VSP accel threshold
    float resetPositions, clampPositionDelta, pad1, pad2;
    float bones[512][16];  // row_major float4x4, row-vector convention: p' = [p 1] * M
};
static_assert(sizeof(SimParamsF) == 160 + 512 * 64, "layout");

template <class T> struct Quat { T x, y, z, w; };

template <class T> struct SimConsts {
    V3<T> wind[4];
    T damping, localStiffness, globalStiffness, globalRange;
    T gravity, timeStep, tipSeparation;
    int lengthIterations;
    T vspCoeff, vspAccelThreshold;
    T reset, clamp;
    T decay;
    const float* bones;  // 512 x 16, converted on read
    bool anyWind;
};

template <class T> static SimConsts<T> load_consts(const SimParamsF* cb) {
    SimConsts<T> c;
    const float* w[4] = {cb->wind, cb->wind1, cb->wind2, cb->wind3};
    for (int i = 0; i < 4; ++i) c.wind[i] = {T(w[i][0]), T(w[i][1]), T(w[i][2])};
    c.anyWind = (cb->wind[0] != 0.0f || cb->wind[1] != 0.0f || cb->wind[2] != 0.0f);
    c.damping = T(cb->shape[0]);
    c.localStiffness = T(cb->shape[1]);
    c.globalStiffness = T(cb->shape[2]);
    c.globalRange = T(cb->shape[3]);
    c.gravity = T(cb->gravTimeTip[0]);
    c.timeStep = T(cb->gravTimeTip[1]);
    c.tipSeparation = T(cb->gravTimeTip[2]);
    c.lengthIterations = cb->simInts[0];
    c.vspCoeff = T(cb->vsp[0]);
    c.vspAccelThreshold = T(cb->vsp[1]);
    c.reset = T(cb->resetPositions);
    c.clamp = T(cb->clampPositionDelta);
    // Integrate(), TressFXSimulation.hlsl:444: exp(-dampingCoeff * g_TimeStep * 60.0f)
    T arg = (-c.damping * c.timeStep) * T(60.0f);
    c.decay = std::exp(arg);
    c.bones = &cb->bones[0][0];
    return c;
}

// ----------------------------------------------------------------------------- hair object view
template <class T> struct Hair {
    int G, n, F;  // guide strands, vertices per strand, follow strands per guide
    T* pos; T* prev; T* prevprev; T* tan;  // float4[Vtot]
    T* sld;                                  // StrandLevelData{skinningQuat, vspQuat, vspTranslation}[Stot]
    const T* init;                           // float4[Vtot] rest positions
    const T* rest;                           // float[Vtot] rest lengths
    const T* followOffset;                   // float4[Stot]
    const T* skin;                           // {float4 boneIndex, float4 boneWeight}[Stot]
};

// ----------------------------------------------------------------------------- quaternion helpers
// MultQuaternionAndVector, TressFXSimulation.hlsl:305-315
template <class T> static inline V3<T> qrot(Quat<T> q, V3<T> v) {
    V3<T> qv = {q.x, q.y, q.z};
    V3<T> uv = cross(qv, v);
    V3<T> uuv = cross(qv, uv);
    uv = uv * (T(2.0f) * q.w);
    uuv = uuv * T(2.0f);
    return (v + uv) + uuv;
}

// NormalizeQuaternion, TressFXSimulation.hlsl:329-342
template <class T> static inline Quat<T> qnormalize(Quat<T> q) {
    T n = q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w;
    if (n < T(1e-10f)) { q.w = T(1.0f); return q; }
    T s = T(1.0f) / std::sqrt(n);
    return {q.x * s, q.y * s, q.z * s, q.w * s};
}

// QuatFromTwoUnitVectors, TressFXSimulation.hlsl:345-363
template <class T> static inline Quat<T> qfrom2(V3<T> u, V3<T> v) {
    T r = T(1.0f) + dot(u, v);
    V3<T> n;
    if (r < T(1e-7f)) {
        r = T(0.0f);
        n = std::fabs(u.x) > std::fabs(u.z) ? V3<T>{-u.y, u.x, T(0.0f)} : V3<T>{T(0.0f), -u.z, u.y};
    } else {
        n = cross(u, v);
    }
    return qnormalize(Quat<T>{n.x, n.y, n.z, r});
}

// MakeQuaternion(float4x4), TressFXSimulation.hlsl:247-288 (m[i][j] = row i, column j)
template <class T> static inline Quat<T> quat_from_matrix(const T m[4][4]) {
    Quat<T> q;
    T trace = m[0][0] + m[1][1] + m[2][2];
    if (trace > T(0.0f)) {
        T r = std::sqrt(trace + T(1.0f));
        q.w = T(0.5f) * r;
        r = T(0.5f) / r;
        q.x = (m[1][2] - m[2][1]) * r;
        q.y = (m[2][0] - m[0][2]) * r;
        q.z = (m[0][1] - m[1][0]) * r;
    } else {
        int i = 0, j = 1, k = 2;
        if (m[1][1] > m[0][0]) { i = 1; j = 2; k = 0; }
        if (m[2][2] > m[i][i]) { i = 2; j = 0; k = 1; }
        T r = std::sqrt(m[i][i] - m[j][j] - m[k][k] + T(1.0f));
        T qq[3];
        qq[i] = T(0.5f) * r;
        r = T(0.5f) / r;
        q.w = (m[j][k] - m[k][j]) * r;
        qq[j] = (m[j][i] + m[i][j]) * r;
        qq[k] = (m[k][i] + m[i][k]) * r;
        q.x = qq[0]; q.y = qq[1]; q.z = qq[2];
    }
    return q;
}

// ApplyVertexBoneSkinning, matrix path, TressFXSimulation.hlsl:550-568
template <class T> static inline V3<T> skin_vertex(V3<T> p, const T* skin, const float* bones, Quat<T>* boneQuat) {
    const T* idx = skin;
    const T* wgt = skin + 4;
    T m[4][4];
    int b0 = ftoi(idx[0]);
    const float* M0 = bones + 16 * b0;
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) m[r][c] = T(M0[4 * r + c]) * wgt[0];
    T wsum = wgt[0];
    for (int i = 1; i < 4; ++i) {
        if (wgt[i] > T(0.0f)) {
            const float* Mi = bones + 16 * ftoi(idx[i]);
            for (int r = 0; r < 4; ++r)
                for (int c = 0; c < 4; ++c) m[r][c] = m[r][c] + T(Mi[4 * r + c]) * wgt[i];
            wsum = wsum + wgt[i];
        }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) m[r][c] = m[r][c] / wsum;
    *boneQuat = quat_from_matrix(m);
    // mul(float4(p,1), M).xyz
    V3<T> o;
    o.x = ((p.x * m[0][0] + p.y * m[1][0]) + p.z * m[2][0]) + T(1.0f) * m[3][0];
    o.y = ((p.x * m[0][1] + p.y * m[1][1]) + p.z * m[2][1]) + T(1.0f) * m[3][1];
    o.z = ((p.x * m[0][2] + p.y * m[1][2]) + p.z * m[2][2]) + T(1.0f) * m[3][2];
    return o;
}

// ----------------------------------------------------------------------------- thread pool
template <class F> static void parallel_for(int64_t count, int threads, F&& fn) {
    if (count <= 0) return;
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    int64_t chunk = std::max<int64_t>(1, (count + threads * 8 - 1) / (threads * 8));
    if (threads == 1 || count <= chunk) { fn(int64_t(0), count); return; }
    std::atomic<int64_t> next{0};
    auto worker = [&]() {
        for (;;) {
            int64_t b = next.fetch_add(chunk);
            if (b >= count) break;
            fn(b, std::min(count, b + chunk));
        }
    };
    std::vector<std::thread> pool;
    int nt = (int)std::min<int64_t>(threads, (count + chunk - 1) / chunk);
    for (int t = 1; t < nt; ++t) pool.emplace_back(worker);
    worker();
    for (auto& th : pool) th.join();
}

// ============================================================================= simulation stages
// IntegrationAndGlobalShapeConstraints, TressFXSimulation.hlsl:609-666 (+ Integrate :440-446,
// UpdateFinalVertexPositions :581-586).  One guide strand per work item.
template <class T> static void stage_integrate(const Hair<T>& h, const SimConsts<T>& c, int64_t g) {
    const int n = h.n;
    const int64_t gs = g * (h.F + 1);
    const T* skin = h.skin + 8 * gs;
    const T grav_y = c.gravity * T(-1.0f);
    const T grav_x = c.gravity * T(0.0f);
    for (int j = 0; j < n; ++j) {
        const int64_t gv = gs * n + j;
        V4<T> initialPos = ld4(h.init, gv);
        Quat<T> bq;
        V3<T> sk = skin_vertex(xyz(initialPos), skin, c.bones, &bq);
        initialPos.x = sk.x; initialPos.y = sk.y; initialPos.z = sk.z;
        V4<T> currentPos = ld4(h.pos, gv);
        V4<T> shared = currentPos;
        V4<T> oldPos = ld4(h.prev, gv);
        if (c.reset != T(0.0f)) { currentPos = initialPos; oldPos = initialPos; }
        if (currentPos.w > T(0.0f)) {
            // curPosition + decay * (curPosition - oldPosition) + force * g_TimeStep * g_TimeStep
            V3<T> cur = xyz(currentPos), old = xyz(oldPos);
            V3<T> force = {grav_x, grav_y, grav_x};
            V3<T> r = (cur + c.decay * (cur - old)) + (force * c.timeStep) * c.timeStep;
            shared.x = r.x; shared.y = r.y; shared.z = r.z;
        } else {
            shared = initialPos;
        }
        if (c.globalStiffness > T(0.0f) && c.globalRange != T(0.0f)) {
            if (shared.w > T(0.0f)) {
                if (T(j) < c.globalRange * T(n)) {
                    V3<T> del = c.globalStiffness * (xyz(initialPos) - xyz(shared));
                    shared.x = shared.x + del.x; shared.y = shared.y + del.y; shared.z = shared.z + del.z;
                }
            }
        }
        st4(h.prevprev, gv, ld4(h.prev, gv));
        st4(h.prev, gv, currentPos);
        st4(h.pos, gv, shared);
    }
}

// CalculateStrandLevelData, TressFXSimulation.hlsl:677-728
template <class T> static void stage_strand_level(const Hair<T>& h, const SimConsts<T>& c, int64_t g) {
    const int64_t gs = g * (h.F + 1);
    const int64_t root = gs * h.n;
    V4<T> oo1 = ld4(h.prevprev, root + 1);
    V4<T> o0 = ld4(h.prev, root), o1 = ld4(h.prev, root + 1);
    V4<T> n0 = ld4(h.pos, root), n1 = ld4(h.pos, root + 1);
    V3<T> u = normalize(xyz(o1) - xyz(o0));
    V3<T> v = normalize(xyz(n1) - xyz(n0));
    Quat<T> rot = qfrom2(u, v);
    V3<T> trans = xyz(n0) - qrot(rot, xyz(o0));
    T vspCoeff = c.vspCoeff;
    // length(pos_new[1] - 2.0 * pos_old[1] + pos_old_old[1]) over all four components
    T ax = (n1.x - T(2.0f) * o1.x) + oo1.x;
    T ay = (n1.y - T(2.0f) * o1.y) + oo1.y;
    T az = (n1.z - T(2.0f) * o1.z) + oo1.z;
    T aw = (n1.w - T(2.0f) * o1.w) + oo1.w;
    T accel = std::sqrt(ax * ax + ay * ay + az * az + aw * aw);
    if (accel > c.vspAccelThreshold) vspCoeff = T(1.0f);
    T* s = h.sld + 12 * gs;
    s[4] = rot.x; s[5] = rot.y; s[6] = rot.z; s[7] = rot.w;
    s[8] = trans.x; s[9] = trans.y; s[10] = trans.z; s[11] = vspCoeff;
    Quat<T> bq;
    (void)skin_vertex(xyz(ld4(h.init, root)), h.skin + 8 * gs, c.bones, &bq);
    s[0] = bq.x; s[1] = bq.y; s[2] = bq.z; s[3] = bq.w;
}

// VelocityShockPropagation, TressFXSimulation.hlsl:739-762
template <class T> static void stage_vsp(const Hair<T>& h, const SimConsts<T>&, int64_t g) {
    const int64_t gs = g * (h.F + 1);
    const T* s = h.sld + 12 * gs;
    Quat<T> q = {s[4], s[5], s[6], s[7]};
    V3<T> t = {s[8], s[9], s[10]};
    T cf = s[11];
    for (int j = 2; j < h.n; ++j) {
        const int64_t gv = gs * h.n + j;
        V3<T> pn = xyz(ld4(h.pos, gv));
        V3<T> po = xyz(ld4(h.prev, gv));
        pn = (T(1.0f) - cf) * pn + cf * (qrot(q, pn) + t);
        po = (T(1.0f) - cf) * po + cf * (qrot(q, po) + t);
        st3(h.pos, gv, pn);
        st3(h.prev, gv, po);
    }
}

// LocalShapeConstraints, TressFXSimulation.hlsl:773-829 (one dispatch = one sweep)
template <class T> static void stage_local_shape(const Hair<T>& h, const SimConsts<T>& c, int64_t g) {
    const int64_t gs = g * (h.F + 1);
    const int64_t root = gs * h.n;
    T stiff = T(0.5f) * std::fmin(c.localStiffness, T(0.95f));
    const T* s = h.sld + 12 * gs;
    Quat<T> bq = {s[0], s[1], s[2], s[3]};
    for (int j = 1; j < h.n - 1; ++j) {
        const int64_t gv = root + j;
        V4<T> pos = ld4(h.pos, gv);
        V4<T> pp1 = ld4(h.pos, gv + 1);
        V4<T> pm1 = ld4(h.pos, gv - 1);
        V3<T> bind = qrot(bq, xyz(ld4(h.init, gv)));
        V3<T> bindp1 = qrot(bq, xyz(ld4(h.init, gv + 1)));
        V3<T> bindm1 = qrot(bq, xyz(ld4(h.init, gv - 1)));
        V3<T> lastVec = xyz(pos) - xyz(pm1);
        V3<T> vecBindPose = bindp1 - bind;
        V3<T> lastVecBindPose = bind - bindm1;
        Quat<T> rotGlobal = qfrom2(normalize(lastVecBindPose), normalize(lastVec));
        V3<T> org = qrot(rotGlobal, vecBindPose) + xyz(pos);
        V3<T> del = stiff * (org - xyz(pp1));
        if (pos.w > T(0.0f)) { pos.x = pos.x - del.x; pos.y = pos.y - del.y; pos.z = pos.z - del.z; }
        if (pp1.w > T(0.0f)) { pp1.x = pp1.x + del.x; pp1.y = pp1.y + del.y; pp1.z = pp1.z + del.z; }
        st3(h.pos, gv, xyz(pos));
        st3(h.pos, gv + 1, xyz(pp1));
    }
}

// ApplyDistanceConstraint + ConstraintMultiplier, TressFXSimulation.hlsl:214-230, 377-387
template <class T> static inline void distance_constraint(V4<T>& p0, V4<T>& p1, T target) {
    V3<T> delta = xyz(p1) - xyz(p0);
    T distance = std::fmax(length(delta), T(1e-7f));
    T stretching = T(1.0f) - target / distance;
    delta = stretching * delta;
    T m0, m1;
    if (p0.w > T(0.0f)) { if (p1.w > T(0.0f)) { m0 = T(0.5f); m1 = T(0.5f); } else { m0 = T(1.0f); m1 = T(0.0f); } }
    else { if (p1.w > T(0.0f)) { m0 = T(0.0f); m1 = T(1.0f); } else { m0 = T(0.0f); m1 = T(0.0f); } }
    V3<T> a = (m0 * delta) * T(1.0f);
    V3<T> b = (m1 * delta) * T(1.0f);
    p0.x = p0.x + a.x; p0.y = p0.y + a.y; p0.z = p0.z + a.z;
    p1.x = p1.x - b.x; p1.y = p1.y - b.y; p1.z = p1.z - b.z;
}

// LengthConstriantsWindAndCollision, TressFXSimulation.hlsl:875-975 (capsules compiled out)
template <class T> static void stage_length_wind(const Hair<T>& h, const SimConsts<T>& c, int64_t g) {
    const int n = h.n;
    const int64_t gs = g * (h.F + 1);
    const int64_t root = gs * n;
    V4<T> sp[64];
    T len[64];
    for (int j = 0; j < n; ++j) { sp[j] = ld4(h.pos, root + j); len[j] = h.rest[root + j]; }
    if (c.anyWind) {
        T a = T((float)(gs % 20)) / T(20.0f);
        V3<T> w = ((a * c.wind[0] + (T(1.0f) - a) * c.wind[1]) + a * c.wind[2]) + (T(1.0f) - a) * c.wind[3];
        V3<T> disp[64];
        for (int j = 2; j < n - 1; ++j) {
            V3<T> v = xyz(sp[j]) - xyz(sp[j + 1]);
            V3<T> force = -cross(cross(v, w), v);
            disp[j] = (force * c.timeStep) * c.timeStep;
        }
        for (int j = 2; j < n - 1; ++j) { sp[j].x = sp[j].x + disp[j].x; sp[j].y = sp[j].y + disp[j].y; sp[j].z = sp[j].z + disp[j].z; }
    }
    const int na = n / 2, nb = (n - 1) / 2;
    for (int it = 0; it < c.lengthIterations; ++it) {
        for (int i = 0; i < na; ++i) distance_constraint(sp[2 * i], sp[2 * i + 1], len[2 * i]);
        for (int i = 0; i < nb; ++i) distance_constraint(sp[2 * i + 1], sp[2 * i + 2], len[2 * i + 1]);
    }
    for (int j = 0; j < n; ++j) {
        const int64_t gv = root + j;
        V4<T> oldPos = ld4(h.prev, gv);
        int ti = (j == n - 1) ? j - 1 : j;
        st3(h.tan, gv, normalize(xyz(sp[ti + 1]) - xyz(sp[ti])));
        V3<T> d = xyz(sp[j]) - xyz(oldPos);
        T speedSqr = dot(d, d);
        if (speedSqr > c.clamp * c.clamp) {
            d = d * ((c.clamp * c.clamp) / speedSqr);
            st3(h.prev, gv, xyz(sp[j]) - d);
        }
        st4(h.pos, gv, sp[j]);
    }
}

// UpdateFollowHairVertices, TressFXSimulation.hlsl:978-1001
template <class T> static void stage_follow(const Hair<T>& h, const SimConsts<T>& c, int64_t g) {
    const int n = h.n, F = h.F;
    const int64_t gs = g * (F + 1);
    for (int j = 0; j < n; ++j) {
        const int64_t gv = gs * n + j;
        V4<T> p = ld4(h.pos, gv);
        V4<T> t = ld4(h.tan, gv);
        for (int i = 0; i < F; ++i) {
            int64_t fv = gv + (int64_t)n * (i + 1);
            int64_t fs = gs + i + 1;
            T factor = c.tipSeparation * (T((float)j) / T((float)n)) + T(1.0f);
            V3<T> off = xyz(ld4(h.followOffset, fs));
            st3(h.pos, fv, xyz(p) + factor * off);
            st4(h.tan, fv, t);
        }
    }
}

// ============================================================================= SDF
struct SdfParamsF {
    float origin[4];
    float cellSize;
    int32_t nx, ny, nz;
};

static inline uint32_t float_flip3(float f) { uint32_t u; std::memcpy(&u, &f, 4); return (u << 1) | (u >> 31); }
static inline uint32_t ifloat_flip3(uint32_t u) { return (u >> 1) | (u << 31); }
static inline uint64_t float_flip3(double f) { uint64_t u; std::memcpy(&u, &f, 8); return (u << 1) | (u >> 63); }
static inline uint64_t ifloat_flip3(uint64_t u) { return (u >> 1) | (u << 63); }
template <class T> struct SdfWord { using type = uint32_t; };
template <> struct SdfWord<double> { using type = uint64_t; };

template <class T> struct Grid {
    V3<T> origin; T cell; int nx, ny, nz;
};
template <class T> static Grid<T> load_grid(const SdfParamsF* p) {
    return {{T(p->origin[0]), T(p->origin[1]), T(p->origin[2])}, T(p->cellSize), p->nx, p->ny, p->nz};
}

// GetSdfCoordinates / GetSdfCellPosition / GetSdfCellIndex, TressFXSDFCollision.hlsl:103-129
template <class T> static inline void sdf_coords(const Grid<T>& g, V3<T> p, int r[3]) {
    V3<T> s = {(p.x - g.origin.x) / g.cell, (p.y - g.origin.y) / g.cell, (p.z - g.origin.z) / g.cell};
    r[0] = ftoi(s.x); r[1] = ftoi(s.y); r[2] = ftoi(s.z);
}
template <class T> static inline V3<T> sdf_cell_pos(const Grid<T>& g, int x, int y, int z) {
    V3<T> c = {T((float)x) * g.cell, T((float)y) * g.cell, T((float)z) * g.cell};
    return c + g.origin;
}

// DistancePointToEdge, TressFXSDFCollision.hlsl:147-159 (the normal output does not reach d)
template <class T> static inline T dist_point_edge(V3<T> p, V3<T> x0, V3<T> x1) {
    V3<T> x10 = x1 - x0;
    T t = dot(x1 - p, x10) / dot(x10, x10);
    t = std::fmax(T(0.0f), std::fmin(t, T(1.0f)));
    V3<T> a = p - (t * x0 + (T(1.0f) - t) * x1);
    return length(a);
}

// SignedDistancePointToTriangle, TressFXSDFCollision.hlsl:163-215
template <class T> static inline T signed_dist_triangle(V3<T> p, V3<T> x0, V3<T> x1, V3<T> x2) {
    T d;
    V3<T> x02 = x0 - x2;
    T l0 = length(x02) + T(1e-30f);
    x02 = x02 / l0;
    V3<T> x12 = x1 - x2;
    T l1 = dot(x12, x02);
    x12 = x12 - l1 * x02;
    T l2 = length(x12) + T(1e-30f);
    x12 = x12 / l2;
    V3<T> px2 = p - x2;
    T b = dot(x12, px2) / l2;
    T a = (dot(x02, px2) - l1 * b) / l0;
    T c = (T(1.0f) - a) - b;
    V3<T> nTri = cross(x1 - x0, x2 - x0);
    T tol = T(1e-8f);
    if (a >= -tol && b >= -tol && c >= -tol) {
        V3<T> nn = p - ((a * x0 + b * x1) + c * x2);
        d = length(nn);
    } else {
        d = dist_point_edge(p, x0, x1);
        T d12 = dist_point_edge(p, x1, x2);
        T d02 = dist_point_edge(p, x0, x2);
        d = std::fmin(d, d12);
        d = std::fmin(d, d02);
    }
    d = (dot(p - x0, nTri) < T(0.0f)) ? -d : d;
    return d;
}

// InitializeSignedDistanceField, TressFXSDFCollision.hlsl:301-312
template <class T> static void sdf_initialize(typename SdfWord<T>::type* sdf, int64_t cells) {
    const auto v = float_flip3(T(1e10f));
    for (int64_t i = 0; i < cells; ++i) sdf[i] = v;
}

// ConstructSignedDistanceField, TressFXSDFCollision.hlsl:329-397 (one triangle)
template <class T> static void sdf_construct_tri(typename SdfWord<T>::type* sdf, const Grid<T>& g, const float* mesh,
                                                 const uint32_t* idx, int64_t t) {
    using W = typename SdfWord<T>::type;
    V3<T> tri[3];
    for (int k = 0; k < 3; ++k) {
        const float* v = mesh + 8 * (int64_t)idx[3 * t + k];
        tri[k] = {T(v[0]), T(v[1]), T(v[2])};
    }
    V3<T> m = {g.cell, g.cell, g.cell};
    V3<T> aabbMin = vmin(tri[0], vmin(tri[1], tri[2])) - m;
    V3<T> aabbMax = vmax(tri[0], vmax(tri[1], tri[2])) + m;
    int lo[3], hi[3];
    sdf_coords(g, aabbMin, lo);
    sdf_coords(g, aabbMax, hi);
    const int dims[3] = {g.nx, g.ny, g.nz};
    for (int k = 0; k < 3; ++k) {
        lo[k] = lo[k] - 1; hi[k] = hi[k] + 1;
        lo[k] = std::max(0, std::min(lo[k], dims[k] - 1));
        hi[k] = std::max(0, std::min(hi[k], dims[k] - 1));
    }
    for (int z = lo[2]; z <= hi[2]; ++z)
        for (int y = lo[1]; y <= hi[1]; ++y)
            for (int x = lo[0]; x <= hi[0]; ++x) {
                int64_t ci = (int64_t)g.nx * g.ny * z + (int64_t)g.nx * y + x;
                T d = signed_dist_triangle(sdf_cell_pos(g, x, y, z), tri[0], tri[1], tri[2]);
                W enc = float_flip3(d);
                W cur = __atomic_load_n(&sdf[ci], __ATOMIC_RELAXED);
                while (enc < cur && !__atomic_compare_exchange_n(&sdf[ci], &cur, enc, true, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
                }
            }
}

// FinalizeSignedDistanceField, TressFXSDFCollision.hlsl:400-412
template <class T> static void sdf_finalize(typename SdfWord<T>::type* sdf, int64_t cells) {
    for (int64_t i = 0; i < cells; ++i) sdf[i] = ifloat_flip3(sdf[i]);
}

template <class T> static inline T as_dist(const typename SdfWord<T>::type* sdf, int64_t i) {
    T f; std::memcpy(&f, &sdf[i], sizeof(T)); return f;
}

template <class T> static inline T lerp(T a, T b, T t) { return a * (T(1.0f) - t) + b * t; }

// GetSignedDistance + TrilinearInterpolate, TressFXSDFCollision.hlsl:414-527
template <class T> static T sdf_lookup(const typename SdfWord<T>::type* sdf, const Grid<T>& g, V3<T> p) {
    int gc[3];
    sdf_coords(g, p, gc);
    if (!(0 <= gc[0] && gc[0] < g.nx - 2) || !(0 <= gc[1] && gc[1] < g.ny - 2) || !(0 <= gc[2] && gc[2] < g.nz - 2))
        return T(1e10f);
    int64_t base = (int64_t)g.nx * g.ny * gc[2] + (int64_t)g.nx * gc[1] + gc[0];
    int64_t X = 1, Y = g.nx, Z = (int64_t)g.ny * g.nx;
    const int64_t off[8] = {0, X, Y, Y + X, Z, Z + X, Z + Y, Z + Y + X};
    T d[8];
    for (int j = 0; j < 8; ++j) {
        d[j] = as_dist<T>(sdf, base + off[j]);
        if (d[j] == T(1e10f)) return T(1e10f);
    }
    V3<T> cp = sdf_cell_pos(g, gc[0], gc[1], gc[2]);
    V3<T> ip = (p - cp) / g.cell;
    T b0 = lerp(lerp(d[0], d[1], ip.x), lerp(d[2], d[3], ip.x), ip.y);
    T b1 = lerp(lerp(d[4], d[5], ip.x), lerp(d[6], d[7], ip.x), ip.y);
    return lerp(b0, b1, ip.z);
}

// CollideHairVerticesWithSdf_forward, TressFXSDFCollision.hlsl:531-595 (one vertex)
template <class T> static void sdf_collide_vertex(const typename SdfWord<T>::type* sdf, const Grid<T>& g, T margin,
                                                  T* pos, T* prev, int n, int64_t v) {
    int local = (int)(v % n);
    if (local == 0 || local == 1) return;
    V4<T> hv = ld4(pos, v);
    V3<T> p = xyz(hv);
    T distance = sdf_lookup(sdf, g, p);
    if (distance > margin) return;
    T h = T(0.1f) * g.cell;
    const V3<T> offs[3] = {{T(1.0f), T(0.0f), T(0.0f)}, {T(0.0f), T(1.0f), T(0.0f)}, {T(0.0f), T(0.0f), T(1.0f)}};
    T fd[3];
    for (int i = 0; i < 3; ++i) fd[i] = sdf_lookup(sdf, g, p + offs[i] * h);
    V3<T> grad = {(fd[0] - distance) / h, (fd[1] - distance) / h, (fd[2] - distance) / h};
    V3<T> nrm = normalize(grad);
    if (distance < margin) {
        V3<T> proj = p + nrm * (margin - distance);
        st3(pos, v, proj);
        st3(prev, v, proj);
    }
}

// CollideHairVerticesWithSdf, TressFXSDFCollision.hlsl:599-715 (one vertex; every vertex of the
// object, roots included): one 8-corner fetch, the gradient by forward or backward differences inside
// the same cell, with h = 0.1 * cellSize added to the cell-normalised coordinates as the shader does.
template <class T> static void sdf_collide_mixed_vertex(const typename SdfWord<T>::type* sdf, const Grid<T>& g, T margin,
                                                        T* pos, T* prev, int64_t v) {
    V4<T> hv = ld4(pos, v);
    V3<T> p = xyz(hv);
    int gc[3];
    sdf_coords(g, p, gc);
    if (!(0 <= gc[0] && gc[0] < g.nx - 2) || !(0 <= gc[1] && gc[1] < g.ny - 2) || !(0 <= gc[2] && gc[2] < g.nz - 2)) return;
    int64_t base = (int64_t)g.nx * g.ny * gc[2] + (int64_t)g.nx * gc[1] + gc[0];
    int64_t X = 1, Y = g.nx, Z = (int64_t)g.ny * g.nx;
    const int64_t off[8] = {0, X, Y, Y + X, Z, Z + X, Z + Y, Z + Y + X};
    T d[8];
    for (int j = 0; j < 8; ++j) {
        d[j] = as_dist<T>(sdf, base + off[j]);
        if (d[j] == T(1e10f)) return;
    }
    auto tri = [&](T x, T y, T z) {
        T b0 = lerp(lerp(d[0], d[1], x), lerp(d[2], d[3], x), y);
        T b1 = lerp(lerp(d[4], d[5], x), lerp(d[6], d[7], x), y);
        return lerp(b0, b1, z);
    };
    V3<T> cp = sdf_cell_pos(g, gc[0], gc[1], gc[2]);
    V3<T> ip = (p - cp) / g.cell;
    T dist = tri(ip.x, ip.y, ip.z);
    T h = T(0.1f) * g.cell;
    V3<T> dir = {(ip.x + h < T(1.0f)) ? T(1.0f) : T(-1.0f), (ip.y + h < T(1.0f)) ? T(1.0f) : T(-1.0f),
                 (ip.z + h < T(1.0f)) ? T(1.0f) : T(-1.0f)};
    V3<T> nd = {tri(ip.x + h * dir.x, ip.y, ip.z), tri(ip.x, ip.y + h * dir.y, ip.z), tri(ip.x, ip.y, ip.z + h * dir.z)};
    V3<T> grad = {(dir.x * (nd.x - dist)) / h, (dir.y * (nd.y - dist)) / h, (dir.z * (nd.z - dist)) / h};
    V3<T> nrm = normalize(grad);
    if (dist < margin) {
        V3<T> proj = p + nrm * (margin - dist);
        st3(pos, v, proj);
        st3(prev, v, proj);
    }
}

// BoneSkinning, src/Shaders/TressFXBoneSkinning.hlsl:57-94 (collision-mesh LBS; one vertex)
static void mesh_skin_vertex(float* out, const float* in, const float* skin, const float* bones, int64_t v) {
    const float* pin = in + 8 * v;
    const float* idx = skin + 8 * v;
    const float* wgt = idx + 4;
    float m[4][4];
    const float* M0 = bones + 16 * ftoi(idx[0]);
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) m[r][c] = M0[4 * r + c] * wgt[0];
    float wsum = wgt[0];
    for (int i = 1; i < 4; ++i) {
        if (wgt[i] > 0.0f) {
            const float* Mi = bones + 16 * ftoi(idx[i]);
            for (int r = 0; r < 4; ++r)
                for (int c = 0; c < 4; ++c) m[r][c] = m[r][c] + Mi[4 * r + c] * wgt[i];
            wsum = wsum + wgt[i];
        }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) m[r][c] = m[r][c] / wsum;
    float* po = out + 8 * v;
    float px = pin[0], py = pin[1], pz = pin[2];
    float nx = pin[4], ny = pin[5], nz = pin[6];
    for (int c = 0; c < 3; ++c) {
        po[c] = ((px * m[0][c] + py * m[1][c]) + pz * m[2][c]) + 1.0f * m[3][c];
        po[4 + c] = ((nx * m[0][c] + ny * m[1][c]) + nz * m[2][c]) + 0.0f * m[3][c];
    }
}

}  // namespace tfxo

// ============================================================================= C interface
using namespace tfxo;

typedef struct tfxo_hair {
    int32_t num_guide_strands, verts_per_strand, follow_per_guide, _pad;
    void* pos; void* prev; void* prevprev; void* tan; void* sld;
    const void* init; const void* rest; const void* follow_offset; const void* skin;
} tfxo_hair;

enum { TFXO_INTEGRATE = 1, TFXO_STRAND_LEVEL = 2, TFXO_VSP = 3, TFXO_LOCAL_SHAPE = 4, TFXO_LENGTH_WIND = 5, TFXO_FOLLOW = 6 };

template <class T> static Hair<T> view(const tfxo_hair* d) {
    Hair<T> h;
    h.G = d->num_guide_strands; h.n = d->verts_per_strand; h.F = d->follow_per_guide;
    h.pos = (T*)d->pos; h.prev = (T*)d->prev; h.prevprev = (T*)d->prevprev; h.tan = (T*)d->tan; h.sld = (T*)d->sld;
    h.init = (const T*)d->init; h.rest = (const T*)d->rest; h.followOffset = (const T*)d->follow_offset; h.skin = (const T*)d->skin;
    return h;
}

template <class T> static int run_stage(int stage, const tfxo_hair* hd, const void* cbv, int threads) {
    if (!hd || !cbv) return 1;
    Hair<T> h = view<T>(hd);
    if (h.n < 3 || h.n > 64 || 64 % h.n != 0 || h.G < 0 || h.F < 0) return 2;
    SimConsts<T> c = load_consts<T>((const SimParamsF*)cbv);
    switch (stage) {
        case TFXO_INTEGRATE: parallel_for(h.G, threads, [&](int64_t b, int64_t e) { for (int64_t g = b; g < e; ++g) stage_integrate(h, c, g); }); break;
        case TFXO_STRAND_LEVEL: parallel_for(h.G, threads, [&](int64_t b, int64_t e) { for (int64_t g = b; g < e; ++g) stage_strand_level(h, c, g); }); break;
        case TFXO_VSP: parallel_for(h.G, threads, [&](int64_t b, int64_t e) { for (int64_t g = b; g < e; ++g) stage_vsp(h, c, g); }); break;
        case TFXO_LOCAL_SHAPE: parallel_for(h.G, threads, [&](int64_t b, int64_t e) { for (int64_t g = b; g < e; ++g) stage_local_shape(h, c, g); }); break;
        case TFXO_LENGTH_WIND: parallel_for(h.G, threads, [&](int64_t b, int64_t e) { for (int64_t g = b; g < e; ++g) stage_length_wind(h, c, g); }); break;
        case TFXO_FOLLOW: parallel_for(h.G, threads, [&](int64_t b, int64_t e) { for (int64_t g = b; g < e; ++g) stage_follow(h, c, g); }); break;
        default: return 1;
    }
    return 0;
}

extern "C" int tfxo_stage_f32(int stage, const tfxo_hair* h, const void* cb, int threads) { return run_stage<float>(stage, h, cb, threads); }
extern "C" int tfxo_stage_f64(int stage, const tfxo_hair* h, const void* cb, int threads) { return run_stage<double>(stage, h, cb, threads); }

// TressFXSimulation::Simulate order (TressFXSimulation.cpp:77-112) for one object:
// integrate, strand level, VSP, local shape x cpu_local_iterations, length/wind, follow.
template <class T> static int run_simulate(const tfxo_hair* h, const void* cb, int cpu_local_iterations, int threads) {
    int stages[] = {TFXO_INTEGRATE, TFXO_STRAND_LEVEL, TFXO_VSP};
    for (int s : stages) if (int r = run_stage<T>(s, h, cb, threads)) return r;
    for (int i = 0; i < cpu_local_iterations; ++i) if (int r = run_stage<T>(TFXO_LOCAL_SHAPE, h, cb, threads)) return r;
    if (int r = run_stage<T>(TFXO_LENGTH_WIND, h, cb, threads)) return r;
    return run_stage<T>(TFXO_FOLLOW, h, cb, threads);
}
extern "C" int tfxo_simulate_f32(const tfxo_hair* h, const void* cb, int it, int threads) { return run_simulate<float>(h, cb, it, threads); }
extern "C" int tfxo_simulate_f64(const tfxo_hair* h, const void* cb, int it, int threads) { return run_simulate<double>(h, cb, it, threads); }

// SDF build = Initialize + Construct + Finalize (TressFXSDFCollision.cpp:95-169).
// sdf: uint32 cells (f32) or uint64 cells (f64); mesh: {float4 position, float4 normal}[Vm].
template <class T> static int run_sdf_build(void* sdfv, const SdfParamsF* gp, const float* mesh, const uint32_t* idx,
                                            int64_t ntri, int threads) {
    using W = typename SdfWord<T>::type;
    if (!sdfv || !gp || (ntri > 0 && (!mesh || !idx))) return 1;
    W* sdf = (W*)sdfv;
    Grid<T> g = load_grid<T>(gp);
    int64_t cells = (int64_t)g.nx * g.ny * g.nz;
    sdf_initialize<T>(sdf, cells);
    parallel_for(ntri, threads, [&](int64_t b, int64_t e) { for (int64_t t = b; t < e; ++t) sdf_construct_tri<T>(sdf, g, mesh, idx, t); });
    sdf_finalize<T>(sdf, cells);
    return 0;
}
extern "C" int tfxo_sdf_build_f32(void* sdf, const void* gp, const float* mesh, const uint32_t* idx, int64_t ntri, int threads) {
    return run_sdf_build<float>(sdf, (const SdfParamsF*)gp, mesh, idx, ntri, threads);
}
extern "C" int tfxo_sdf_build_f64(void* sdf, const void* gp, const float* mesh, const uint32_t* idx, int64_t ntri, int threads) {
    return run_sdf_build<double>(sdf, (const SdfParamsF*)gp, mesh, idx, ntri, threads);
}
// Construct only, into a caller-initialised grid (no init / finalize); for per-kernel checks.
extern "C" int tfxo_sdf_construct_f32(uint32_t* sdf, const void* gp, const float* mesh, const uint32_t* idx, int64_t ntri, int threads) {
    Grid<float> g = load_grid<float>((const SdfParamsF*)gp);
    parallel_for(ntri, threads, [&](int64_t b, int64_t e) { for (int64_t t = b; t < e; ++t) sdf_construct_tri<float>(sdf, g, mesh, idx, t); });
    return 0;
}
extern "C" float tfxo_signed_distance_triangle_f32(const float* p, const float* x0, const float* x1, const float* x2) {
    return signed_dist_triangle<float>({p[0], p[1], p[2]}, {x0[0], x0[1], x0[2]}, {x1[0], x1[1], x1[2]}, {x2[0], x2[1], x2[2]});
}
extern "C" uint32_t tfxo_float_flip3(float f) { return float_flip3(f); }
extern "C" uint32_t tfxo_ifloat_flip3(uint32_t u) { return ifloat_flip3(u); }

// CollideHairVerticesWithSdf_forward over all Vtot vertices; margin = collisionMargin * cellSize
// (TressFXSDFCollision.cpp:194).
template <class T> static int run_collide(const void* sdfv, const SdfParamsF* gp, float margin, const tfxo_hair* hd, int threads) {
    using W = typename SdfWord<T>::type;
    if (!sdfv || !gp || !hd) return 1;
    Hair<T> h = view<T>(hd);
    Grid<T> g = load_grid<T>(gp);
    int64_t vtot = (int64_t)h.G * (h.F + 1) * h.n;
    const W* sdf = (const W*)sdfv;
    parallel_for(vtot, threads, [&](int64_t b, int64_t e) {
        for (int64_t v = b; v < e; ++v) sdf_collide_vertex<T>(sdf, g, T(margin), h.pos, h.prev, h.n, v);
    });
    return 0;
}
extern "C" int tfxo_sdf_collide_f32(const void* sdf, const void* gp, float margin, const tfxo_hair* h, int threads) {
    return run_collide<float>(sdf, (const SdfParamsF*)gp, margin, h, threads);
}
extern "C" int tfxo_sdf_collide_f64(const void* sdf, const void* gp, float margin, const tfxo_hair* h, int threads) {
    return run_collide<double>(sdf, (const SdfParamsF*)gp, margin, h, threads);
}

template <class T> static int run_collide_mixed(const void* sdfv, const SdfParamsF* gp, float margin, const tfxo_hair* hd,
                                                int threads) {
    using W = typename SdfWord<T>::type;
    if (!sdfv || !gp || !hd) return 1;
    Hair<T> h = view<T>(hd);
    Grid<T> g = load_grid<T>(gp);
    int64_t vtot = (int64_t)h.G * (h.F + 1) * h.n;
    const W* sdf = (const W*)sdfv;
    parallel_for(vtot, threads, [&](int64_t b, int64_t e) {
        for (int64_t v = b; v < e; ++v) sdf_collide_mixed_vertex<T>(sdf, g, T(margin), h.pos, h.prev, v);
    });
    return 0;
}
extern "C" int tfxo_sdf_collide_mixed_f32(const void* sdf, const void* gp, float margin, const tfxo_hair* h, int threads) {
    return run_collide_mixed<float>(sdf, (const SdfParamsF*)gp, margin, h, threads);
}

// Collision-mesh bone skinning (BoneSkinning kernel, one thread per mesh vertex).
// in/out: {float4 position, float4 normal}[Vm] (w copied from in); skin: {float4 idx, float4 w}[Vm].
extern "C" int tfxo_mesh_skin_f32(float* out, const float* in, const float* skin, const float* bones, int64_t nverts, int threads) {
    if (!out || !in || !skin || !bones) return 1;
    parallel_for(nverts, threads, [&](int64_t b, int64_t e) {
        for (int64_t v = b; v < e; ++v) {
            out[8 * v + 3] = in[8 * v + 3];
            out[8 * v + 7] = in[8 * v + 7];
            mesh_skin_vertex(out, in, skin, bones, v);
        }
    });
    return 0;
}

// ================================================================================================
// Strand quad expansion: GetExpandedTressFXVert / GetExpandedTressFXShadowVert
// (src/Shaders/TressFXStrands.hlsl), the vertex-shader arithmetic that turns each hair vertex into
// two camera-facing quad vertices.  Conventions: Safe_normalize (TressFXUtilities.hlsl:104-119) with
// rcp = the IEEE reciprocal; lerp(x, y, s) = x + s (y - x); mul(M, v) summed left to right over the
// row; the albedo texture is white (texture sampling is graphics).
namespace {
struct F2 { float x, y; };
struct F3x { float x, y, z; };
inline F3x sub3(F3x a, F3x b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline F3x scl3(F3x a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline F3x add3(F3x a, F3x b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline F3x safe3(F3x v) {
    const float len = std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
    if (!(len >= 1e-7f)) return {0.0f, 0.0f, 0.0f};
    return scl3(v, 1.0f / len);
}
inline F2 safe2(F2 v) {
    const float len = std::sqrt(v.x * v.x + v.y * v.y);
    if (!(len >= 1e-7f)) return {0.0f, 0.0f};
    const float r = 1.0f / len;
    return {v.x * r, v.y * r};
}
inline void mulMv(const float* M, const float v[4], float o[4]) {
    for (int r = 0; r < 4; ++r) o[r] = ((M[4 * r] * v[0] + M[4 * r + 1] * v[1]) + M[4 * r + 2] * v[2]) + M[4 * r + 3] * v[3];
}
}  // namespace

extern "C" int tfxo_expand_strands(const float* pos, const float* tan, int64_t vtot, const float* fp, const int* ip,
                                   const float* eye, const float* win, const float* VP, int shadow, float* out) {
    if (!pos || !tan || !fp || !ip || !eye || !win || !VP || !out || ip[0] < 2) return 1;
    const int n = ip[0], thinTip = ip[1];
    const F3x eyeV = {eye[0], eye[1], eye[2]};
    for (int64_t id = 0; id < 2 * vtot; ++id) {
        const uint32_t vid = (uint32_t)id;
        const int64_t index = vid / 2;
        const F3x v = {pos[4 * index], pos[4 * index + 1], pos[4 * index + 2]};
        const F3x t = {tan[4 * index], tan[4 * index + 1], tan[4 * index + 2]};
        const uint32_t inStrand = (uint32_t)(index % n);
        const float fraction = (float)inStrand / (float)(n - 1);
        const float ratio = thinTip > 0 ? 1.0f + fraction * (fp[10] - 1.0f) : 1.0f;
        const F3x vv = safe3(sub3(v, eyeV));
        const F3x right = safe3({t.y * vv.z - t.z * vv.y, t.z * vv.x - t.x * vv.z, t.x * vv.y - t.y * vv.x});
        const float r4[4] = {right.x, right.y, right.z, 0.0f};
        float pr[4];
        mulMv(VP, r4, pr);
        const F2 projRight = safe2({pr[0], pr[1]});
        const float expandPixels = shadow ? 1.0f : 0.71f;
        const F3x p0 = add3(v, scl3(scl3(scl3(right, -1.0f), ratio), fp[11]));
        const F3x p1 = add3(v, scl3(scl3(scl3(right, 1.0f), ratio), fp[11]));
        const float h0[4] = {p0.x, p0.y, p0.z, 1.0f}, h1[4] = {p1.x, p1.y, p1.z, 1.0f};
        float e0[4], e1[4];
        mulMv(VP, h0, e0);
        mulMv(VP, h1, e1);
        const bool odd = (vid & 1u) != 0;
        const float fDir = odd ? -1.0f : 1.0f;
        const float* sel = odd ? e0 : e1;
        const float offv[4] = {(projRight.x * expandPixels) / win[1], (projRight.y * expandPixels) / win[1], 0.0f, 0.0f};
        float* o = out + 16 * id;
        for (int c = 0; c < 4; ++c) o[c] = sel[c] + (fDir * offv[c]) * sel[3];
        for (int c = 4; c < 16; ++c) o[c] = 0.0f;
        if (shadow) continue;
        const float uvx = odd ? 0.0f : 1.0f;
        o[4] = t.x; o[5] = t.y; o[6] = t.z; o[7] = uvx;
        const float w0 = std::fmax(e0[3], 1e-7f), w1 = std::fmax(e1[3], 1e-7f);
        o[8] = e0[0] / w0; o[9] = e0[1] / w0; o[10] = e1[0] / w1; o[11] = e1[1] / w1;
        const F3x root = {1.0f * fp[0], 1.0f * fp[1], 1.0f * fp[2]};
        const F3x tip = {fp[4], fp[5], fp[6]};
        const float rootRange = 1.0f - fp[8];
        const F3x col = fraction > rootRange ? add3(root, scl3(sub3(tip, root), fraction)) : root;
        o[12] = col.x; o[13] = col.y; o[14] = col.z; o[15] = fraction;
    }
    return 0;
}

// ============================================================================ marching cubes
// RunMarchingCubesOnSdf (TressFXMarchingCubes.hlsl:147-280) over every cell in index order -- the order
// in which a one-thread-at-a-time dispatch appends -- after InitializeMCVertices (:127-145).  The
// tables are the caller's (the shader reads them from buffers).  Output: {position, normal} as 8
// floats per vertex; *counter = every cube's reservation, as the shader's InterlockedAdd counter.
namespace {
const int kMcCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 0, 1}, {0, 0, 1}, {0, 1, 0}, {1, 1, 0}, {1, 1, 1}, {0, 1, 1}};
const int kMcEdge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6}, {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
}  // namespace

extern "C" int tfxo_marching_cubes_f32(const float* sdf, const SdfParamsF* g, float iso, const int32_t* edgeTable,
                                       const int32_t* triTable, int maxVerts, float* out, int32_t* counter) {
    if (!sdf || !g || !edgeTable || !triTable || (!out && maxVerts > 0) || !counter || maxVerts < 0) return 1;
    for (int i = 0; i < 256 * 16; ++i)
        if (triTable[i] < -1 || triTable[i] > 11) return 2;
    std::memset(out, 0, (size_t)maxVerts * 8 * sizeof(float));
    const int X = g->nx, Y = g->ny, Z = g->nz;
    const int64_t total = (int64_t)X * Y * Z;
    int64_t count = 0;
    for (int64_t idx = 0; idx < total; ++idx) {
        const int z = (int)(idx / ((int64_t)X * Y)), rem = (int)(idx % ((int64_t)X * Y));
        const int y = rem / X, x = rem % X;
        if (!(x < X - 1) || !(y < Y - 1) || !(z < Z - 1)) continue;
        float pos[8][3], s[8];
        for (int k = 0; k < 8; ++k) {
            const int cx = x + kMcCorner[k][0], cy = y + kMcCorner[k][1], cz = z + kMcCorner[k][2];
            pos[k][0] = (float)cx * g->cellSize;
            pos[k][1] = (float)cy * g->cellSize;
            pos[k][2] = (float)cz * g->cellSize;
            pos[k][0] = pos[k][0] + g->origin[0];
            pos[k][1] = pos[k][1] + g->origin[1];
            pos[k][2] = pos[k][2] + g->origin[2];
            s[k] = sdf[(int64_t)X * Y * cz + (int64_t)X * cy + cx];
        }
        int cfg = 0;
        for (int k = 0; k < 8; ++k)
            if (s[k] < iso) cfg |= 1 << k;
        if (!edgeTable[cfg]) continue;
        float v[12][3] = {};
        for (int e = 0; e < 12; ++e) {
            if (!(edgeTable[cfg] & (1 << e))) continue;
            const int a = kMcEdge[e][0], b = kMcEdge[e][1];
            const float interp = (iso - s[a]) / (s[b] - s[a]);
            for (int d = 0; d < 3; ++d) v[e][d] = pos[a][d] + (pos[b][d] - pos[a][d]) * interp;
        }
        int nv = 0;
        while (nv < 16 && triTable[cfg * 16 + nv] != -1) ++nv;
        const int64_t offset = count;
        count += nv;
        if (!(offset + nv < maxVerts)) continue;
        for (int t = 0; t < nv / 3; ++t) {
            const float* p[3];
            for (int c = 0; c < 3; ++c) p[c] = v[triTable[cfg * 16 + 3 * t + c]];
            const float a[3] = {p[1][0] - p[0][0], p[1][1] - p[0][1], p[1][2] - p[0][2]};
            const float b[3] = {p[2][0] - p[0][0], p[2][1] - p[0][1], p[2][2] - p[0][2]};
            const float n[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
            const float inv = 1.0f / std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
            for (int c = 0; c < 3; ++c) {
                float* o = out + 8 * (offset + 3 * t + c);
                o[0] = p[c][0]; o[1] = p[c][1]; o[2] = p[c][2]; o[3] = 0.f;
                o[4] = n[0] * inv; o[5] = n[1] * inv; o[6] = n[2] * inv; o[7] = 0.f;
            }
        }
    }
    *counter = (int32_t)count;
    return 0;
}

// ============================================================================================
// Host-side constants: TressFXSimulationSettings -> TressFXSimulationParams header.
// Restates TressFXSettings.h:38-56 (defaults), TressFXHairObject.cpp:380-437
// (UpdateSimulationParameters), :172-235 (SetWindCorner, SetWind) and the pieces of src/Math the
// wind uses (Vector3 Cross / Length / Normalize, Vector3D.h:70-75 and Vector3D.cpp:48-62;
// Quaternion SetRotation / operator* , Quaternion.cpp:79-89, 262-284), in float, in the
// reference's operation order.  The reference is a Windows build whose unqualified sin / pow / asin
// on floats are the float functions; they are called as sinf / powf / asinf here.
// ============================================================================================
struct SettingsF {   // TressFXSimulationSettings, declaration order (TressFXSettings.h:59-87)
    float vspCoeff, vspAccelThreshold, localStiffness;
    int32_t localIterations;
    float globalStiffness, globalRange;
    int32_t lengthIterations;
    float damping, gravity, tipSeparation, windMagnitude, windDirection[3], windAngle, clampPositionDelta;
};
static_assert(sizeof(SettingsF) == 64, "layout");

namespace host {

struct Vec { float x, y, z; };
struct Rot { float x, y, z, w; };   // quaternion, identity = (0, 0, 0, 1)

static Vec cross(Vec a, Vec b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
static float length(Vec a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }
static void normalize_in_place(Vec& a) {   // leaves a zero vector unchanged
    const float d = sqrtf(a.x * a.x + a.y * a.y + a.z * a.z);
    if (d == 0) return;
    a.x = a.x / d; a.y = a.y / d; a.z = a.z / d;
}
static Rot axis_angle(Vec axis, float angle) {
    const float h = 0.5f * angle;
    const float s = sinf(h);
    return {s * axis.x, s * axis.y, s * axis.z, cosf(h)};
}
static Rot compose(Rot a, Rot b) {   // a * b
    Rot q;
    q.w = a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z;
    q.x = a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y;
    q.y = a.w * b.y + a.y * b.w + a.z * b.x - a.x * b.z;
    q.z = a.w * b.z + a.z * b.w + a.x * b.y - a.y * b.x;
    return q;
}
static Vec rotate(Rot q, Vec v) {   // v + 2w (q x v) + 2 q x (q x v)
    const Vec qv{q.x, q.y, q.z};
    Vec uv = cross(qv, v);
    Vec uuv = cross(qv, uv);
    const float s = 2.0f * q.w;
    uv = {uv.x * s, uv.y * s, uv.z * s};
    uuv = {uuv.x * 2.0f, uuv.y * 2.0f, uuv.z * 2.0f};
    const Vec a{v.x + uv.x, v.y + uv.y, v.z + uv.z};
    return {a.x + uuv.x, a.y + uuv.y, a.z + uuv.z};
}

// one edge of the wind pyramid (SetWindCorner)
static void wind_corner(Rot toWind, Vec axis, float coneAngle, float wM, float out[4]) {
    const Vec d = rotate(compose(toWind, axis_angle(axis, coneAngle)), Vec{1.0f, 0.0f, 0.0f});
    out[0] = d.x * wM;
    out[1] = d.y * wM;
    out[2] = d.z * wM;
    out[3] = 0.0f;
}

static void set_wind(SimParamsF* p, const float dir[3], float magnitude, int frame) {
    const float wM = magnitude * (powf(sinf(frame * 0.01f), 2.0f) + 0.5f);
    Vec w{dir[0], dir[1], dir[2]};
    normalize_in_place(w);
    Vec axis = cross(Vec{1.0f, 0.0f, 0.0f}, w);
    Rot toWind{0.0f, 0.0f, 0.0f, 1.0f};
    const float angle = asinf(length(axis));
    if (angle > 0.001) {   // a double comparison, as in the reference
        normalize_in_place(axis);
        toWind = axis_angle(axis, angle);
    }
    const float cone = 40.f * 3.14159265359f / 180;   // DEG_TO_RAD2(40.f)
    wind_corner(toWind, Vec{0, 1.0f, 0}, cone, wM, p->wind);
    wind_corner(toWind, Vec{0, -1.0f, 0}, cone, wM, p->wind1);
    wind_corner(toWind, Vec{0, 0, 1.0f}, cone, wM, p->wind2);
    wind_corner(toWind, Vec{0, 0, -1.0f}, cone, wM, p->wind3);
}

}  // namespace host

extern "C" void tfxo_settings_default(SettingsF* s) {
    s->vspCoeff = 0.8f;
    s->vspAccelThreshold = 1.4f;
    s->localStiffness = 0.9f;
    s->localIterations = 2;
    s->globalStiffness = 0.0f;
    s->globalRange = 0.0f;
    s->lengthIterations = 2;
    s->damping = 0.08f;
    s->gravity = 0.0f;
    s->tipSeparation = 0.0f;
    s->windMagnitude = 0.0f;
    s->windDirection[0] = 1.0f;
    s->windDirection[1] = 0.0f;
    s->windDirection[2] = 0.0f;
    s->windAngle = 3.1415926f / 180.0f * 40.0f;
    s->clampPositionDelta = 20.f;
}

// UpdateSimulationParameters on the constant block of the current frame; the reset flag is set for
// frames 0 and 1 and otherwise left as the block holds it.  Returns m_CPULocalShapeIterations.
extern "C" int tfxo_fill_sim_params(const SettingsF* s, float timeStep, int n, int F, int frame, SimParamsF* p) {
    p->vsp[0] = s->vspCoeff;
    p->vsp[1] = s->vspAccelThreshold;
    p->shape[0] = s->damping;
    p->shape[1] = s->localStiffness;
    p->shape[2] = s->globalStiffness;
    p->shape[3] = s->globalRange;
    p->gravTimeTip[0] = s->gravity;
    p->gravTimeTip[1] = timeStep;
    p->simInts[2] = 0;                 // SetCollision(false)
    p->counts[0] = 64 / n;             // TRESSFX_SIM_THREAD_GROUP_SIZE / n
    p->counts[2] = n;
    p->counts[1] = F;
    p->gravTimeTip[2] = s->tipSeparation;
    p->clampPositionDelta = 20.0f;
    int cpuIterations;
    if (n >= 64) {                     // TRESSFX_MIN_VERTS_PER_STRAND_FOR_GPU_ITERATION
        p->simInts[1] = s->localIterations;
        cpuIterations = 1;
    } else {
        p->simInts[1] = 1;
        cpuIterations = s->localIterations;
    }
    p->simInts[0] = s->lengthIterations;
    host::set_wind(p, s->windDirection, s->windMagnitude, frame);
    if (frame < 2) p->resetPositions = 1.0f;
    return cpuIterations;
}
