/*
 * Bit-compatible C restatement of the structs Reina shares between its host code and its shaders.
 *
 *   InstanceProperties     <- polyglot/raytrace.h:18-41   (120 bytes; `bool interpNormals` is 4 bytes,
 *                                                         as in GLSL scalar layout and in the C++ layout
 *                                                         where the bool is followed by 3 padding bytes)
 *   RtPushConsts           <- polyglot/raytrace.h:43-54   (160 bytes; mat4 column-major, glm convention)
 *   BloomPushConsts        <- polyglot/bloom.h:4-8
 *   TonemappingPushConsts  <- polyglot/tonemapping.h:4-6
 *   EmissiveInstanceData   <- src/scene/Instances.h:15-27 (`InstanceData`, alignas(16), 112 bytes)
 *
 * The reference builds these with glm types; here they use plain float arrays so that any C caller can
 * fill them.  Field order, meaning and byte offsets are unchanged.
 */
#ifndef REINA_POLYGLOT_H
#define REINA_POLYGLOT_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct InstanceProperties {
    uint32_t indicesOffset;
    float albedo[3];
    float emission[3];
    uint32_t tbnsIndicesOffset;
    uint32_t texIndicesOffset;   /* 0xFFFFFFFF: the model has no texture coordinates */
    float roughness;
    float ior;
    uint32_t interpNormals;      /* GLSL bool */
    float absorption;
    int32_t textureID;
    int32_t normalMapTexID;
    int32_t bumpMapTexID;
    uint32_t cullBackface;
    float anisotropic;
    float subsurface;
    float clearcoatGloss;
    float sheenTint[3];
    float specularTint[3];
    float metallic;
    float clearcoat;
    float specularTransmission;
    float sheen;
} InstanceProperties;

typedef struct RtPushConsts {
    float invView[16];           /* column-major: element (row r, column c) is invView[c*4 + r] */
    float invProjection[16];
    uint32_t sampleBatch;
    float totalEmissiveWeight;
    float focusDist;
    float defocusMultiplier;
    float directClamp;
    float indirectClamp;         /* read from config.toml but used by no shader of the reference */
    uint32_t samplesPerPixel;
    uint32_t maxBounces;
} RtPushConsts;

typedef struct BloomPushConsts {
    float radius;                /* percent of the image side; also the Gaussian sigma in taps */
    float threshold;
    float intensity;
} BloomPushConsts;

typedef struct TonemappingPushConsts {
    float exposure;
} TonemappingPushConsts;

typedef struct EmissiveInstanceData {
    float transform[16];         /* column-major */
    uint32_t materialOffset;
    uint32_t cdfRangeStart;
    uint32_t cdfRangeEnd;
    uint32_t indexOffset;
    float emission[3];
    float weight;
    float area;
    uint32_t cullBackface;       /* GLSL bool */
    float padding[2];
} EmissiveInstanceData;

#ifdef __cplusplus
}  /* extern "C" */
static_assert(sizeof(InstanceProperties) == 120, "InstanceProperties must stay 120 bytes");
static_assert(sizeof(RtPushConsts) == 160, "RtPushConsts must stay 160 bytes");
static_assert(sizeof(EmissiveInstanceData) == 112, "EmissiveInstanceData must stay 112 bytes");
#endif

#endif  /* REINA_POLYGLOT_H */
