// ref_math_shim.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Exposes the reference's own host-compiled math (tdc-lib/include/gpumath.h and
// tdc-lib/include/windowing.h, included from the reference checkout, not copied)
// through a C ABI so that tests can compare the oracle's FP64 restatement with
// the reference's FP32 functions on the same inputs. Built by oracle/build.py
// into oracle/_ref/.
#include <vector_types.h>

#include "gpumath.h"
#include "windowing.h"

extern "C" {

float ref_norm3(float x, float y, float z) { return hdNorm3df(x, y, z); }

void ref_float2_add(const float *a, const float *b, float *out)
{
    float2 r = float2{a[0], a[1]} + float2{b[0], b[1]};
    out[0] = r.x;
    out[1] = r.y;
}

void ref_float3_sub(const float *a, const float *b, float *out)
{
    float3 r = float3{a[0], a[1], a[2]} - float3{b[0], b[1], b[2]};
    out[0] = r.x;
    out[1] = r.y;
    out[2] = r.z;
}

float ref_dot3(const float *a, const float *b)
{
    return v3_dot(float3{a[0], a[1], a[2]}, float3{b[0], b[1], b[2]});
}

// Quaternions are (w, x, y, z), stored in float4 (x, y, z, w) as the reference does.
void ref_q_conj(const float *q, float *out)
{
    float4 r = q_conj(float4{q[0], q[1], q[2], q[3]});
    out[0] = r.x;
    out[1] = r.y;
    out[2] = r.z;
    out[3] = r.w;
}

void ref_q_prod(const float *a, const float *b, float *out)
{
    float4 r = q_prod(float4{a[0], a[1], a[2], a[3]}, float4{b[0], b[1], b[2], b[3]});
    out[0] = r.x;
    out[1] = r.y;
    out[2] = r.z;
    out[3] = r.w;
}

void ref_q_rot(const float *q, const float *v, float *out)
{
    float3 r = q_rot(float4{q[0], q[1], q[2], q[3]}, float3{v[0], v[1], v[2]});
    out[0] = r.x;
    out[1] = r.y;
    out[2] = r.z;
}

float ref_doppler_centroid(const float *vel, const float *ant, float lambda)
{
    return dopplerCentroid(float3{vel[0], vel[1], vel[2]}, float3{ant[0], ant[1], ant[2]}, lambda);
}

float ref_doppler_freq(const float *pos, const float *vel, const float *tgt, float lambda)
{
    return dopplerFreq(float3{pos[0], pos[1], pos[2]}, float3{vel[0], vel[1], vel[2]},
                       float3{tgt[0], tgt[1], tgt[2]}, lambda);
}

float ref_doppler_window(float f_dop, float f_center, float bw, int taper)
{
    return dopplerWindow(f_dop, f_center, bw, taper != 0);
}

float ref_range_window_a() { return RANGE_WINDOW_A_PARAMETER; }
float ref_azimuth_window_a() { return AZIMUTH_WINDOW_A_PARAMETER; }
int ref_pri_chunksize() { return static_cast<int>(PRI_CHUNKSIZE); }

}  // extern "C"
