// types.h -- data layouts shared by the host code and the kernels (no
// device code, so the host translation units can include it).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/ptgpu.h"

namespace ptgpu {

// ---------------------------------------------------------------------------
// Traversal layouts
//
// Node (64 B, four 16-byte loads): both children's boxes plus child refs.
//   q0 = (L.min_x, L.max_x, L.min_y, L.max_y)
//   q1 = (L.min_z, L.max_z, R.min_x, R.max_x)
//   q2 = (R.min_y, R.max_y, R.min_z, R.max_z)
//   q3 = (left, right, left_count, right_count) as ints: count 0 means an
//        internal node index, count > 0 a leaf range [ref, ref+count) of prims.
// Prim (48 B, three 16-byte loads), in leaf order:
//   triangle: (p1, TRI) (e1, 0) (e2, 0) with e1 = p2-p1, e2 = p3-p1
//   sphere:   (p, SPH)  (rad*rad, rad, 0, 0) (0)
// ---------------------------------------------------------------------------
// 4-wide node (128 B, eight 16-byte loads), one per binary node; a 4-wide
// node's slots are the binary node's children, an internal child replaced by
// its own two children.  Traversal starts at node 0 and follows slot refs,
// so only the nodes at even binary depth are ever visited.
//   q0..q5 = min_x[4], max_x[4], min_y[4], max_y[4], min_z[4], max_z[4]
//   q6     = ref[4]   (internal: binary node index; leaf: first prim)
//   q7     = count[4] (0: internal, > 0: leaf prim count, -1: empty slot)
struct TraceView {
    const float4 *nodes;     // internal nodes (may be null when the root is a leaf)
    const float4 *nodes4;    // 4-wide nodes (null: traverse the binary nodes)
    const float4 *prims;     // prims in traversal order
    const int32_t *prim_id;  // traversal-order prim -> shape id
    int32_t accel;           // PTGPU_ACCEL_*
    int32_t root_count;      // 0: root is internal node 0; >0: root is a leaf range
    int32_t root_first;
    int32_t n_shapes;
    const float *root_box;   // device: min_x,max_x,min_y,max_y,min_z,max_z of the root
    int32_t *error_flags;    // bit 0: stack overflow
};

struct LightRec {            // one emitter, in index order (SampleLights)
    float4 a;                // tri: (p1, type)   sphere: (p, type)
    float4 b;                // tri: (e1, area)   sphere: (rad, -, -, area)
    float4 c;                // tri: (e2, 0)
    float4 e;                // emission (e.xyz, 0)
};

struct Material {            // per shape
    float4 c_refl;           // (c.xyz, refl as float bits)
    float4 e_type;           // (e.xyz, type as float bits)
};

}  // namespace ptgpu
