// Host-side constant preparation of the C ABI: simulation settings -> constant block
// (TressFXHairObject::UpdateSimulationParameters / SetWind) and SDF grid sizing
// (TressFXSDFCollision ctor / UpdateSDFGrid).  Pure host arithmetic in float, evaluated in the
// reference's order (built with -ffp-contract=off); no device is touched.
#include <climits>
#include <cmath>
#include <cstring>

#include "../../include/tressfx_gb300.h"

namespace {

// The subset of the reference's host math used by SetWind (src/Math/Vector3D.*, Quaternion.*).
struct Vec3 {
    float x, y, z;
    Vec3 cross(const Vec3& v) const { return {y * v.z - z * v.y, z * v.x - x * v.z, x * v.y - y * v.x}; }
    float length() const { return std::sqrt(x * x + y * y + z * z); }
    // Vector3::Normalize, Vector3D.cpp:48-62
    Vec3& normalize() {
        float d = std::sqrt(x * x + y * y + z * z);
        if (d == 0) return *this;
        x = x / d; y = y / d; z = z / d;
        return *this;
    }
};

struct Quat {
    float x = 0, y = 0, z = 0, w = 1;
    // Quaternion::SetRotation(axis, angle), Quaternion.cpp:79-89
    void set_rotation(const Vec3& axis, float angle) {
        float halfAng = 0.5f * angle;
        float sinHalf = std::sin(halfAng);
        w = std::cos(halfAng);
        x = sinHalf * axis.x; y = sinHalf * axis.y; z = sinHalf * axis.z;
    }
    // Quaternion::operator*(Quaternion), Quaternion.cpp:262-272
    Quat operator*(const Quat& o) const {
        Quat q;
        q.w = w * o.w - x * o.x - y * o.y - z * o.z;
        q.x = w * o.x + x * o.w + y * o.z - z * o.y;
        q.y = w * o.y + y * o.w + z * o.x - x * o.z;
        q.z = w * o.z + z * o.w + x * o.y - y * o.x;
        return q;
    }
    // Quaternion::operator*(Vector3), Quaternion.cpp:274-284
    Vec3 operator*(const Vec3& v) const {
        Vec3 qv{x, y, z};
        Vec3 uv = qv.cross(v);
        Vec3 uuv = qv.cross(uv);
        float s = 2.0f * w;
        uv = {uv.x * s, uv.y * s, uv.z * s};
        uuv = {uuv.x * 2.0f, uuv.y * 2.0f, uuv.z * 2.0f};
        Vec3 a{v.x + uv.x, v.y + uv.y, v.z + uv.z};
        return {a.x + uuv.x, a.y + uuv.y, a.z + uuv.z};
    }
};

// SetWindCorner, TressFXHairObject.cpp:172-185
void set_wind_corner(const Quat& rotFromXAxisToWindDir, Vec3 rotAxis, float angle, float wM, float out[4]) {
    const Vec3 XAxis{1.0f, 0.0f, 0.0f};
    Quat rot;
    rot.set_rotation(rotAxis, angle);
    Vec3 nd = (rotFromXAxisToWindDir * rot) * XAxis;
    out[0] = nd.x * wM;
    out[1] = nd.y * wM;
    out[2] = nd.z * wM;
    out[3] = 0;
}

// TressFXHairObject::SetWind, TressFXHairObject.cpp:191-235
void set_wind(tfx_sim_params* p, const float dir[3], float windMag, int frame) {
    float s = std::sin((float)frame * 0.01f);
    float wM = windMag * (std::pow(s, 2.0f) + 0.5f);
    Vec3 windDirN{dir[0], dir[1], dir[2]};
    windDirN.normalize();
    Vec3 XAxis{1.0f, 0.0f, 0.0f};
    Vec3 xCrossW = XAxis.cross(windDirN);
    Quat rotFromXAxisToWindDir;  // identity
    float angle = std::asin(xCrossW.length());
    if ((double)angle > 0.001) rotFromXAxisToWindDir.set_rotation(xCrossW.normalize(), angle);
    const float MATH_PI2 = 3.14159265359f;
    float angleToWideWindCone = 40.f * MATH_PI2 / 180;
    set_wind_corner(rotFromXAxisToWindDir, Vec3{0, 1.0f, 0}, angleToWideWindCone, wM, p->wind);
    set_wind_corner(rotFromXAxisToWindDir, Vec3{0, -1.0f, 0}, angleToWideWindCone, wM, p->wind1);
    set_wind_corner(rotFromXAxisToWindDir, Vec3{0, 0, 1.0f}, angleToWideWindCone, wM, p->wind2);
    set_wind_corner(rotFromXAxisToWindDir, Vec3{0, 0, -1.0f}, angleToWideWindCone, wM, p->wind3);
}

}  // namespace

extern "C" int tfx_sim_settings_default(tfx_sim_settings* s) {
    if (!s) return TFX_ERR_INVALID_ARGUMENT;
    // TressFXSimulationSettings(), TressFXSettings.h:38-56
    s->vsp_coeff = 0.8f;
    s->vsp_accel_threshold = 1.4f;
    s->local_constraint_stiffness = 0.9f;
    s->local_constraints_iterations = 2;
    s->global_constraint_stiffness = 0.0f;
    s->global_constraints_range = 0.0f;
    s->length_constraints_iterations = 2;
    s->damping = 0.08f;
    s->gravity_magnitude = 0.0f;
    s->tip_separation = 0.0f;
    s->wind_magnitude = 0.0f;
    s->wind_direction[0] = 1.0f;
    s->wind_direction[1] = 0.0f;
    s->wind_direction[2] = 0.0f;
    s->wind_angle_radians = 3.1415926f / 180.0f * 40.0f;
    s->clamp_position_delta = 20.f;
    return TFX_OK;
}

// TressFXHairObject::UpdateSimulationParameters, TressFXHairObject.cpp:380-437
extern "C" int tfx_fill_sim_params(tfx_sim_params* p, const tfx_sim_settings* s, float timeStep, int n, int F, int frame,
                                   int32_t* cpuLocalIterations) {
    if (!p || !s || n <= 0 || n > TFX_THREAD_GROUP_SIZE || F < 0) return TFX_ERR_INVALID_ARGUMENT;
    p->vsp[0] = s->vsp_coeff;
    p->vsp[1] = s->vsp_accel_threshold;
    p->shape[0] = s->damping;
    p->shape[1] = s->local_constraint_stiffness;
    p->shape[2] = s->global_constraint_stiffness;
    p->shape[3] = s->global_constraints_range;
    p->grav_time_tip[0] = s->gravity_magnitude;
    p->grav_time_tip[1] = timeStep;
    p->sim_ints[2] = 0;  // SetCollision(false)
    p->counts[0] = TFX_THREAD_GROUP_SIZE / n;
    p->counts[2] = n;
    p->counts[1] = F;
    p->grav_time_tip[2] = s->tip_separation;
    p->clamp_position_delta = 20.0f;  // hard-coded by the reference, :397
    int cpuIters;
    if (n >= 64) {  // TRESSFX_MIN_VERTS_PER_STRAND_FOR_GPU_ITERATION
        p->sim_ints[1] = s->local_constraints_iterations;
        cpuIters = 1;
    } else {
        p->sim_ints[1] = 1;
        cpuIters = s->local_constraints_iterations;
    }
    p->sim_ints[0] = s->length_constraints_iterations;
    set_wind(p, s->wind_direction, s->wind_magnitude, frame);
    if (frame < 2) p->reset_positions = 1.0f;
    if (cpuLocalIterations) *cpuLocalIterations = cpuIters;
    return TFX_OK;
}

// TressFXSDFCollision ctor, TressFXSDFCollision.cpp:38-75
extern "C" int tfx_sdf_grid_from_bbox(const float bmin_in[3], const float bmax_in[3], int numCellsInX, tfx_sdf_grid* grid,
                                      float* padding, int64_t* allocCells) {
    if (!bmin_in || !bmax_in || !grid || numCellsInX <= 0) return TFX_ERR_INVALID_ARGUMENT;
    float bmin[3] = {bmin_in[0], bmin_in[1], bmin_in[2]};
    float bmax[3] = {bmax_in[0], bmax_in[1], bmax_in[2]};
    float cell = (bmax[0] - bmin[0]) / numCellsInX;
    if (!(cell > 0.0f)) return TFX_ERR_INVALID_ARGUMENT;
    int numExtraPaddingCells = (int)(0.8f * (float)numCellsInX);
    float pad = numExtraPaddingCells * cell;
    // UpdateSDFGrid(bmin, bmax): origin = bmin - padding
    for (int k = 0; k < 3; ++k) grid->origin[k] = bmin[k] - pad;
    grid->origin[3] = 0.0f;
    for (int k = 0; k < 3; ++k) { bmin[k] -= pad; bmax[k] += pad; }
    grid->cell_size = cell;
    grid->num_cells_x = (int)((bmax[0] - bmin[0]) / cell);
    grid->num_cells_y = (int)((bmax[1] - bmin[1]) / cell);
    grid->num_cells_z = (int)((bmax[2] - bmin[2]) / cell);
    if (padding) *padding = pad;
    if (allocCells) {
        const float m = 1.4f;
        int total = (int)(m * grid->num_cells_x * grid->num_cells_y * grid->num_cells_z);
        *allocCells = total < INT_MAX ? total : INT_MAX;
    }
    return TFX_OK;
}

// TressFXSDFCollision::UpdateSDFGrid, TressFXSDFCollision.cpp:88-93
extern "C" int tfx_sdf_grid_origin(const float bmin[3], float padding, tfx_sdf_grid* grid) {
    if (!bmin || !grid) return TFX_ERR_INVALID_ARGUMENT;
    for (int k = 0; k < 3; ++k) grid->origin[k] = bmin[k] - padding;
    grid->origin[3] = 0.0f;
    return TFX_OK;
}
