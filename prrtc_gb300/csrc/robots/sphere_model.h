// pRRTC sphere collision model as plain-C tables.  Generated by
// prrtc_gb300/robots/codegen.py from the fitted model; do not edit.
// Max |sphere centre - reference float64 FK|: 0.000e+00 m
#pragma once
#include "model_types.h"

enum {
    kSphereDof = 3,
    kSphereNumJoints = 3,
    kSphereNumSpheres = 1,
    kSphereNumEnvGroups = 1,
    kSphereNumEnvLeaves = 1,
    kSphereNumSelfGroups = 0,
    kSphereNumSelfPairs = 0,
    kSphereNumSchedule = 1,
};

static const prrtc_joint_def kSphereJoints[] = {
    {0, -1, 0, {0.0f, 0.0f, 1.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f}},
    {1, 0, 0, {0.0f, 0.0f, 1.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f}},
    {2, 1, 0, {0.0f, 0.0f, 1.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f}},
};
static const prrtc_sphere_def kSphereSpheres[] = {
    {2, 0.0f, 0.0f, 0.0f, 1.0f},
};
static const prrtc_group_def kSphereEnvGroups[] = {
    {-1, -1, 0, 1},  /* sphere */
};
static const short kSphereEnvLeaves[] = {
    0,
};
static const prrtc_group_def kSphereSelfGroups[] = {{-1, -1, 0, 0}};
static const short kSphereSelfPairs[][2] = {{0, 0}};
static const prrtc_sched_def kSphereSchedule[] = {
    {0, 0},
};
