// Plain-C description of a robot collision model (shared by the CUDA code
// generator's tables and the CPU oracle).  See prrtc_gb300/robots/extract.py
// for how the tables are derived from pRRTC's generated checkers.
#pragma once

// One joint: config index q, parent joint's config index (-1 = world),
// revolute (1: rotation by q about local z) or prismatic (0: translation by q
// along local z), and F, the fixed 3x4 row-major transform from the parent
// joint's frame to this joint's frame (applied before the joint motion).
typedef struct {
    int q;
    int parent;
    int revolute;
    float F[12];
} prrtc_joint_def;

// One collision sphere: frame = config index of the joint it rides on
// (-1 = world), centre (x, y, z) in that frame, radius r.
typedef struct {
    int frame;
    float x, y, z, r;
} prrtc_sphere_def;

// A gated group of the checker.  Environment group: gate_a = gating sphere
// (-1 = none), gate_b unused; leaves are [first, first+count) of the robot's
// leaf list.  Self group: (gate_a, gate_b) = gating sphere pair; leaf pairs
// are [first, first+count) of the robot's pair list.
typedef struct {
    int gate_a;
    int gate_b;
    int first;
    int count;
} prrtc_group_def;

// The checker's evaluation order: kind 0 = environment group, 1 = self group.
typedef struct {
    int kind;
    int index;
} prrtc_sched_def;
