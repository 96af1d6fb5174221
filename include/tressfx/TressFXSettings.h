// TressFXSimulationSettings (src/TressFX/TressFXSettings.h:35-87): same members, same defaults.
#pragma once

#include "TressFXCommon.h"

class TressFXSimulationSettings {
public:
    TressFXSimulationSettings()
        : m_vspCoeff(0.8f),
          m_vspAccelThreshold(1.4f),
          m_localConstraintStiffness(0.9f),
          m_localConstraintsIterations(2),
          m_globalConstraintStiffness(0.0f),
          m_globalConstraintsRange(0.0f),
          m_lengthConstraintsIterations(2),
          m_damping(0.08f),
          m_gravityMagnitude(0.0f),
          m_tipSeparation(0.0f),
          m_windMagnitude(0),
          m_windAngleRadians(3.1415926f / 180.0f * 40.0f),
          m_clampPositionDelta(20.f) {
        m_windDirection[0] = 1.0f;
        m_windDirection[1] = 0.0f;
        m_windDirection[2] = 0.0f;
    }

    float m_vspCoeff;
    float m_vspAccelThreshold;
    float m_localConstraintStiffness;
    int m_localConstraintsIterations;
    float m_globalConstraintStiffness;
    float m_globalConstraintsRange;
    int m_lengthConstraintsIterations;
    float m_damping;
    float m_gravityMagnitude;
    float m_tipSeparation;
    float m_windMagnitude;
    float m_windDirection[3];
    float m_windAngleRadians;
    float m_clampPositionDelta;

    // The same values as the C ABI's tfx_sim_settings.
    tfx_sim_settings ToC() const {
        tfx_sim_settings s;
        s.vsp_coeff = m_vspCoeff;
        s.vsp_accel_threshold = m_vspAccelThreshold;
        s.local_constraint_stiffness = m_localConstraintStiffness;
        s.local_constraints_iterations = m_localConstraintsIterations;
        s.global_constraint_stiffness = m_globalConstraintStiffness;
        s.global_constraints_range = m_globalConstraintsRange;
        s.length_constraints_iterations = m_lengthConstraintsIterations;
        s.damping = m_damping;
        s.gravity_magnitude = m_gravityMagnitude;
        s.tip_separation = m_tipSeparation;
        s.wind_magnitude = m_windMagnitude;
        s.wind_direction[0] = m_windDirection[0];
        s.wind_direction[1] = m_windDirection[1];
        s.wind_direction[2] = m_windDirection[2];
        s.wind_angle_radians = m_windAngleRadians;
        s.clamp_position_delta = m_clampPositionDelta;
        return s;
    }
};
