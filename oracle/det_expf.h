/*
 * exp(x) in FP32 by Cody-Waite range reduction (x = k ln2 + r, |r| <= ln2/2, ln2
 * split in a 16-bit head and a tail so k * head is exact) and a degree-7 Taylor
 * polynomial in Horner form, scaled by 2^k in two exact steps.  Plain IEEE
 * multiply/add only (compile with -ffp-contract=off), so the frame kernel on the
 * GPU evaluates the identical sequence; at most 2 ulp from exp(x).  Shared by the
 * oracle (C) and the checker build of the reference's frame helpers (C++).
 */
#ifndef GCA_DET_EXPF_H
#define GCA_DET_EXPF_H
#include <math.h>
#include <stdint.h>
#include <string.h>

static inline float gca_det_expf(float x)
{
    if (x != x)
        return x;
    if (x > 88.72283935546875f)
        return INFINITY;
    if (x < -103.972084045410156f)
        return 0.0f;
    const float kf = rintf(x * 1.44269502162933349609f);
    const float r = (x - kf * 0.693145751953125f) - kf * 1.428606765330187045e-06f;
    float p = 1.0f / 5040.0f;
    p = p * r + 1.0f / 720.0f;
    p = p * r + 1.0f / 120.0f;
    p = p * r + 1.0f / 24.0f;
    p = p * r + 1.0f / 6.0f;
    p = p * r + 0.5f;
    p = p * r + 1.0f;
    p = p * r + 1.0f;
    const int k = (int)kf;
    const int k1 = k / 2, k2 = k - k / 2;
    const uint32_t ua = (uint32_t)(k1 + 127) << 23, ub = (uint32_t)(k2 + 127) << 23;
    float a, b;
    memcpy(&a, &ua, 4);
    memcpy(&b, &ub, 4);
    return (p * a) * b;
}
#endif
