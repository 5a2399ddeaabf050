// pRRTC baxter collision model as plain-C tables.  Generated by
// prrtc_gb300/robots/codegen.py from the fitted model; do not edit.
// Max |sphere centre - reference float64 FK|: 2.281e-07 m
#pragma once
#include "model_types.h"

enum {
    kBaxterDof = 14,
    kBaxterNumJoints = 14,
    kBaxterNumSpheres = 100,
    kBaxterNumEnvGroups = 33,
    kBaxterNumEnvLeaves = 75,
    kBaxterNumSelfGroups = 355,
    kBaxterNumSelfPairs = 1925,
    kBaxterNumSchedule = 388,
};

static const prrtc_joint_def kBaxterJoints[] = {
    {0, -1, 1, {1.0f, 0.0f, 0.0f, 0.06402719105656993f, 0.0f, 1.0f, 0.0f, -0.2590274105593823f, 0.0f, 0.0f, 1.0f, 0.0f}},
    {7, -1, 1, {1.0f, 0.0f, 0.0f, 0.0640271646137819f, 0.0f, 1.0f, 0.0f, 0.25902741114481653f, 0.0f, 0.0f, 1.0f, 0.0f}},
    {1, 0, 1, {0.7071054305970537f, 0.0f, 0.7071081317734618f, 0.048790253257584584f, -0.7071081317734613f, 0.0f, 0.7071054305970532f, -0.048790425302413565f, 0.0f, -1.0f, 0.0f, 0.3999759462029193f}},
    {8, 7, 1, {0.7071054321986613f, 0.0f, -0.70710813017186f, 0.04879026697041319f, 0.7071081301718597f, 0.0f, 0.7071054321986613f, 0.048790439230984195f, 0.0f, -1.0f, 0.0f, 0.39997594557256444f}},
    {2, 1, 1, {0.0f, 0.0f, 1.0f, 0.0f, 0.0f, -1.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f}},
    {9, 8, 1, {0.0f, 0.0f, 1.0f, 0.0f, 0.0f, -1.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f}},
    {3, 2, 1, {0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 1.0f, 0.0f, -0.069f, -1.0f, 0.0f, 0.0f, 0.36442f}},
    {10, 9, 1, {0.0f, 0.0f, 1.0f, 0.0f, 0.0f, -1.0f, 0.0f, -0.069f, 1.0f, 0.0f, 0.0f, 0.36442f}},
    {4, 3, 1, {0.0f, 0.0f, -1.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f}},
    {11, 10, 1, {0.0f, 0.0f, 1.0f, 0.0f, 0.0f, -1.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f}},
    {5, 4, 1, {0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 1.0f, 0.0f, -0.01f, -1.0f, 0.0f, 0.0f, 0.37429f}},
    {12, 11, 1, {0.0f, 0.0f, 1.0f, 0.0f, 0.0f, -1.0f, 0.0f, -0.01f, 1.0f, 0.0f, 0.0f, 0.37429f}},
    {6, 5, 1, {0.0f, 0.0f, -1.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f}},
    {13, 12, 1, {0.0f, 0.0f, 1.0f, 0.0f, 0.0f, -1.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f}},
};
static const prrtc_sphere_def kBaxterSpheres[] = {
    {-1, 0.0640272f, 0.2590274f, 0.304626f, 0.175f},
    {-1, 0.0f, 0.0f, -0.6f, 0.5f},
    {-1, 0.0640272f, 0.2590274f, 0.379626f, 0.1f},
    {-1, 0.0640272f, 0.2590274f, 0.229626f, 0.1f},
    {-1, 0.0640272f, -0.2590274f, 0.304626f, 0.175f},
    {-1, 0.0640272f, -0.2590274f, 0.379626f, 0.1f},
    {-1, 0.0640272f, -0.2590274f, 0.229626f, 0.1f},
    {-1, -0.044f, 0.0f, 0.222f, 0.409f},
    {-1, -0.025f, -0.1f, 0.1f, 0.25f},
    {-1, -0.025f, 0.1f, 0.1f, 0.25f},
    {-1, -0.065f, 0.0f, 0.4f, 0.23f},
    {-1, 0.04f, 0.0f, 0.686f, 0.2f},
    {0, 0.04879028520505446f, -0.04879045040186303f, 0.399976f, 0.1f},
    {2, 0.0f, 0.01f, 0.212000055454857f, 0.19f},
    {2, 0.0f, 0.02f, 0.3220000674981451f, 0.08f},
    {2, 0.0f, 0.01f, 0.212000055454857f, 0.08f},
    {1, 0.102f, 0.0f, 0.0f, 0.08f},
    {2, 0.0f, -0.069f, 0.3644200653880031f, 0.1f},
    {4, 0.0f, 0.0f, 0.21359007982510253f, 0.19f},
    {3, -0.10359006850922525f, 0.0f, 0.0f, 0.08f},
    {4, 0.0f, 0.0f, 0.32359009114097986f, 0.08f},
    {4, 0.0f, 0.0f, 0.21359007982510253f, 0.08f},
    {4, 0.0f, -0.01f, 0.3742900956291598f, 0.1f},
    {5, 0.0f, 0.0f, 0.03f, 0.07f},
    {5, 0.0f, 0.0f, -0.03f, 0.07f},
    {6, 0.0f, 0.0f, 0.1009750975804744f, 0.105f},
    {6, 0.0f, 0.0f, 0.13597510118098088f, 0.07f},
    {6, 0.0f, 0.0f, 0.07597509500868416f, 0.08f},
    {6, 0.0f, -0.01f, 0.2095251080197772f, 0.05f},
    {7, 0.04879031164784249f, 0.04879044981642877f, 0.399976f, 0.1f},
    {9, 0.0f, 0.01f, 0.21200005419330953f, 0.19f},
    {9, 0.0f, 0.02f, 0.3220000662365976f, 0.08f},
    {9, 0.0f, 0.01f, 0.21200005419330953f, 0.08f},
    {8, 0.102f, 0.0f, 0.0f, 0.08f},
    {9, 0.0f, -0.069f, 0.36442006412645567f, 0.1f},
    {11, 0.0f, 0.0f, 0.21359007856355516f, 0.19f},
    {10, 0.10359006724767789f, 0.0f, 0.0f, 0.08f},
    {11, 0.0f, 0.0f, 0.32359008987943244f, 0.08f},
    {11, 0.0f, 0.0f, 0.21359007856355516f, 0.08f},
    {11, 0.0f, -0.01f, 0.3742900943676124f, 0.1f},
    {12, 0.0f, 0.0f, 0.03f, 0.07f},
    {12, 0.0f, 0.0f, -0.03f, 0.07f},
    {13, 0.0f, 0.0f, 0.10097509631892698f, 0.105f},
    {13, 0.0f, 0.0f, 0.13597509991943335f, 0.07f},
    {13, 0.0f, 0.0f, 0.07597509374713673f, 0.08f},
    {13, 0.0f, -0.01f, 0.20952510675822977f, 0.05f},
    {13, 0.0f, 0.0f, 0.25452511211486295f, 0.06f},
    {13, 0.02f, 0.0f, 0.2545251116616718f, 0.04f},
    {13, -0.02f, 0.0f, 0.254525112568054f, 0.04f},
    {13, 0.069333f, 0.005f, 0.2825251137879189f, 0.027f},
    {13, 0.081333f, 0.005f, 0.2825251135160043f, 0.015f},
    {13, 0.057333f, 0.005f, 0.2825251140598334f, 0.015f},
    {13, 0.086333f, 0.0f, 0.3245251173596089f, 0.032f},
    {13, 0.086583f, 0.0f, 0.30452511529651183f, 0.012f},
    {13, 0.086583f, 0.0f, 0.32452511735394396f, 0.012f},
    {13, 0.086583f, 0.0f, 0.3445251194113761f, 0.012f},
    {13, 0.082583f, 0.0f, 0.3722251223515579f, 0.028f},
    {13, 0.082083f, -0.01f, 0.38222512266419295f, 0.014f},
    {13, 0.082083f, 0.01f, 0.38222512411901455f, 0.014f},
    {13, 0.082083f, 0.01f, 0.3622251220615823f, 0.014f},
    {13, 0.082083f, -0.01f, 0.3622251206067608f, 0.014f},
    {13, -0.069333f, -0.005f, 0.2825251162026172f, 0.025f},
    {13, -0.059333f, -0.005f, 0.2825251159760217f, 0.015f},
    {13, -0.079333f, -0.005f, 0.28252511642921263f, 0.015f},
    {13, -0.08633305081909415f, 0.0f, 0.3245251212721425f, 0.032f},
    {13, -0.086583f, 0.0f, 0.3045251192203753f, 0.012f},
    {13, -0.08658305082662687f, 0.0f, 0.3245251212778075f, 0.012f},
    {13, -0.08658305182826298f, 0.0f, 0.34452512333523966f, 0.012f},
    {13, -0.08258305309500669f, 0.0f, 0.37222512609414515f, 0.028f},
    {13, -0.08208305285334605f, -0.01f, 0.38222512638412065f, 0.014f},
    {13, -0.08208305430817309f, 0.01f, 0.38222512783894214f, 0.014f},
    {13, -0.08208305330653698f, 0.01f, 0.36222512578151f, 0.014f},
    {13, -0.08208305185170994f, -0.01f, 0.3622251243266885f, 0.014f},
    {6, 0.0f, 0.0f, 0.2545251133764104f, 0.06f},
    {6, 0.02f, 0.0f, 0.2545251137843012f, 0.04f},
    {6, -0.02f, 0.0f, 0.25452511296851954f, 0.04f},
    {6, 0.069333f, 0.005f, 0.2825251180345354f, 0.027f},
    {6, 0.081333f, 0.005f, 0.28252511827926985f, 0.015f},
    {6, 0.057333f, 0.005f, 0.28252511778980094f, 0.015f},
    {6, 0.086333f, 0.0f, 0.3245251223381448f, 0.032f},
    {6, 0.086583f, 0.0f, 0.30452512028581125f, 0.012f},
    {6, 0.086583f, 0.0f, 0.3245251223432435f, 0.012f},
    {6, 0.086583f, 0.0f, 0.3445251244006756f, 0.012f},
    {6, 0.082583f, 0.0f, 0.3722251271686412f, 0.028f},
    {6, 0.082083f, -0.01f, 0.38222512745974924f, 0.014f},
    {6, 0.082083f, 0.01f, 0.3822251289145707f, 0.014f},
    {6, 0.082083f, 0.01f, 0.3622251268571386f, 0.014f},
    {6, 0.082083f, -0.01f, 0.3622251254023171f, 0.014f},
    {6, -0.069333f, -0.005f, 0.2825251144790957f, 0.025f},
    {6, -0.059333f, -0.005f, 0.282525114683041f, 0.015f},
    {6, -0.079333f, -0.005f, 0.28252511427515015f, 0.015f},
    {6, -0.086333f, 0.0f, 0.32452511881670154f, 0.032f},
    {6, -0.086583f, 0.0f, 0.3045251167541707f, 0.012f},
    {6, -0.086583f, 0.0f, 0.32452511881160295f, 0.012f},
    {6, -0.086583f, 0.0f, 0.3445251208690351f, 0.012f},
    {6, -0.082583f, 0.0f, 0.37222512380015693f, 0.028f},
    {6, -0.082083f, -0.01f, 0.38222512411165943f, 0.014f},
    {6, -0.082083f, 0.01f, 0.382225125566481f, 0.014f},
    {6, -0.082083f, 0.01f, 0.3622251235090488f, 0.014f},
    {6, -0.082083f, -0.01f, 0.3622251220542273f, 0.014f},
};
static const prrtc_group_def kBaxterEnvGroups[] = {
    {0, -1, 0, 2},  /* left_upper_shoulder */
    {4, -1, 2, 2},  /* right_upper_shoulder */
    {7, -1, 4, 3},  /* torso */
    {-1, -1, 7, 1},  /*  */
    {-1, -1, 8, 1},  /*  */
    {-1, -1, 9, 1},  /*  */
    {13, -1, 10, 3},  /* right_upper_elbow */
    {-1, -1, 13, 1},  /*  */
    {18, -1, 14, 3},  /* right_upper_forearm */
    {22, -1, 17, 2},  /* right_lower_forearm */
    {25, -1, 19, 2},  /* right_wrist */
    {-1, -1, 21, 1},  /*  */
    {-1, -1, 22, 1},  /*  */
    {30, -1, 23, 3},  /* left_upper_elbow */
    {-1, -1, 26, 1},  /*  */
    {35, -1, 27, 3},  /* left_upper_forearm */
    {39, -1, 30, 2},  /* left_lower_forearm */
    {42, -1, 32, 2},  /* left_wrist */
    {-1, -1, 34, 1},  /*  */
    {46, -1, 35, 2},  /* left_gripper_base */
    {49, -1, 37, 2},  /* l_gripper_l_finger */
    {52, -1, 39, 3},  /* l_gripper_l_finger_2 */
    {56, -1, 42, 4},  /* l_gripper_l_finger_tip */
    {61, -1, 46, 2},  /* l_gripper_r_finger */
    {64, -1, 48, 3},  /* l_gripper_r_finger_2 */
    {68, -1, 51, 4},  /* l_gripper_r_finger_tip */
    {73, -1, 55, 2},  /* right_gripper_base */
    {76, -1, 57, 2},  /* r_gripper_l_finger */
    {79, -1, 59, 3},  /* r_gripper_l_finger_2 */
    {83, -1, 62, 4},  /* r_gripper_l_finger_tip */
    {88, -1, 66, 2},  /* r_gripper_r_finger */
    {91, -1, 68, 3},  /* r_gripper_r_finger_2 */
    {95, -1, 71, 4},  /* r_gripper_r_finger_tip */
};
static const short kBaxterEnvLeaves[] = {
    2, 3, 5, 6, 8, 9, 10, 1, 11, 12, 14, 15, 16, 17, 19, 20,
    21, 23, 24, 26, 27, 28, 29, 31, 32, 33, 34, 36, 37, 38, 40, 41,
    43, 44, 45, 47, 48, 50, 51, 53, 54, 55, 57, 58, 59, 60, 62, 63,
    65, 66, 67, 69, 70, 71, 72, 74, 75, 77, 78, 80, 81, 82, 84, 85,
    86, 87, 89, 90, 92, 93, 94, 96, 97, 98, 99,
};
static const prrtc_group_def kBaxterSelfGroups[] = {
    {0, 1, 0, 2},  /* left_upper_shoulder vs. pedestal */
    {11, 17, 2, 1},  /* head vs. right_lower_elbow */
    {7, 17, 3, 3},  /* torso vs. right_lower_elbow */
    {11, 18, 6, 3},  /* head vs. right_upper_forearm */
    {18, 1, 9, 3},  /* right_upper_forearm vs. pedestal */
    {4, 18, 12, 6},  /* right_upper_shoulder vs. right_upper_forearm */
    {7, 18, 18, 9},  /* torso vs. right_upper_forearm */
    {11, 22, 27, 2},  /* head vs. right_lower_forearm */
    {22, 0, 29, 4},  /* right_lower_forearm vs. left_upper_shoulder */
    {22, 1, 33, 2},  /* right_lower_forearm vs. pedestal */
    {4, 22, 35, 4},  /* right_upper_shoulder vs. right_lower_forearm */
    {7, 22, 39, 6},  /* torso vs. right_lower_forearm */
    {11, 25, 45, 2},  /* head vs. right_wrist */
    {12, 25, 47, 2},  /* right_lower_shoulder vs. right_wrist */
    {13, 25, 49, 6},  /* right_upper_elbow vs. right_wrist */
    {4, 25, 55, 4},  /* right_upper_shoulder vs. right_wrist */
    {25, 0, 59, 4},  /* right_wrist vs. left_upper_shoulder */
    {25, 1, 63, 2},  /* right_wrist vs. pedestal */
    {7, 25, 65, 6},  /* torso vs. right_wrist */
    {11, 28, 71, 1},  /* head vs. right_hand */
    {28, 0, 72, 2},  /* right_hand vs. left_upper_shoulder */
    {28, 1, 74, 1},  /* right_hand vs. pedestal */
    {12, 28, 75, 1},  /* right_lower_shoulder vs. right_hand */
    {13, 28, 76, 3},  /* right_upper_elbow vs. right_hand */
    {4, 28, 79, 2},  /* right_upper_shoulder vs. right_hand */
    {7, 28, 81, 3},  /* torso vs. right_hand */
    {28, 29, 84, 1},  /* right_hand vs. left_lower_shoulder */
    {17, 29, 85, 1},  /* right_lower_elbow vs. left_lower_shoulder */
    {22, 29, 86, 2},  /* right_lower_forearm vs. left_lower_shoulder */
    {18, 29, 88, 3},  /* right_upper_forearm vs. left_lower_shoulder */
    {25, 29, 91, 2},  /* right_wrist vs. left_lower_shoulder */
    {28, 30, 93, 3},  /* right_hand vs. left_upper_elbow */
    {17, 30, 96, 3},  /* right_lower_elbow vs. left_upper_elbow */
    {22, 30, 99, 6},  /* right_lower_forearm vs. left_upper_elbow */
    {18, 30, 105, 9},  /* right_upper_forearm vs. left_upper_elbow */
    {25, 30, 114, 6},  /* right_wrist vs. left_upper_elbow */
    {11, 34, 120, 1},  /* head vs. left_lower_elbow */
    {28, 34, 121, 1},  /* right_hand vs. left_lower_elbow */
    {17, 34, 122, 1},  /* right_lower_elbow vs. left_lower_elbow */
    {22, 34, 123, 2},  /* right_lower_forearm vs. left_lower_elbow */
    {12, 34, 125, 1},  /* right_lower_shoulder vs. left_lower_elbow */
    {13, 34, 126, 3},  /* right_upper_elbow vs. left_lower_elbow */
    {18, 34, 129, 3},  /* right_upper_forearm vs. left_lower_elbow */
    {25, 34, 132, 2},  /* right_wrist vs. left_lower_elbow */
    {7, 34, 134, 3},  /* torso vs. left_lower_elbow */
    {11, 35, 137, 3},  /* head vs. left_upper_forearm */
    {35, 1, 140, 3},  /* left_upper_forearm vs. pedestal */
    {0, 35, 143, 6},  /* left_upper_shoulder vs. left_upper_forearm */
    {28, 35, 149, 3},  /* right_hand vs. left_upper_forearm */
    {17, 35, 152, 3},  /* right_lower_elbow vs. left_upper_forearm */
    {22, 35, 155, 6},  /* right_lower_forearm vs. left_upper_forearm */
    {12, 35, 161, 3},  /* right_lower_shoulder vs. left_upper_forearm */
    {13, 35, 164, 9},  /* right_upper_elbow vs. left_upper_forearm */
    {18, 35, 173, 9},  /* right_upper_forearm vs. left_upper_forearm */
    {25, 35, 182, 6},  /* right_wrist vs. left_upper_forearm */
    {7, 35, 188, 9},  /* torso vs. left_upper_forearm */
    {11, 39, 197, 2},  /* head vs. left_lower_forearm */
    {39, 1, 199, 2},  /* left_lower_forearm vs. pedestal */
    {0, 39, 201, 4},  /* left_upper_shoulder vs. left_lower_forearm */
    {28, 39, 205, 2},  /* right_hand vs. left_lower_forearm */
    {17, 39, 207, 2},  /* right_lower_elbow vs. left_lower_forearm */
    {22, 39, 209, 4},  /* right_lower_forearm vs. left_lower_forearm */
    {12, 39, 213, 2},  /* right_lower_shoulder vs. left_lower_forearm */
    {13, 39, 215, 6},  /* right_upper_elbow vs. left_lower_forearm */
    {18, 39, 221, 6},  /* right_upper_forearm vs. left_lower_forearm */
    {4, 39, 227, 4},  /* right_upper_shoulder vs. left_lower_forearm */
    {25, 39, 231, 4},  /* right_wrist vs. left_lower_forearm */
    {7, 39, 235, 6},  /* torso vs. left_lower_forearm */
    {11, 42, 241, 2},  /* head vs. left_wrist */
    {29, 42, 243, 2},  /* left_lower_shoulder vs. left_wrist */
    {30, 42, 245, 6},  /* left_upper_elbow vs. left_wrist */
    {0, 42, 251, 4},  /* left_upper_shoulder vs. left_wrist */
    {42, 1, 255, 2},  /* left_wrist vs. pedestal */
    {28, 42, 257, 2},  /* right_hand vs. left_wrist */
    {17, 42, 259, 2},  /* right_lower_elbow vs. left_wrist */
    {22, 42, 261, 4},  /* right_lower_forearm vs. left_wrist */
    {12, 42, 265, 2},  /* right_lower_shoulder vs. left_wrist */
    {13, 42, 267, 6},  /* right_upper_elbow vs. left_wrist */
    {18, 42, 273, 6},  /* right_upper_forearm vs. left_wrist */
    {4, 42, 279, 4},  /* right_upper_shoulder vs. left_wrist */
    {25, 42, 283, 4},  /* right_wrist vs. left_wrist */
    {7, 42, 287, 6},  /* torso vs. left_wrist */
    {11, 45, 293, 1},  /* head vs. left_hand */
    {45, 1, 294, 1},  /* left_hand vs. pedestal */
    {29, 45, 295, 1},  /* left_lower_shoulder vs. left_hand */
    {30, 45, 296, 3},  /* left_upper_elbow vs. left_hand */
    {0, 45, 299, 2},  /* left_upper_shoulder vs. left_hand */
    {28, 45, 301, 1},  /* right_hand vs. left_hand */
    {17, 45, 302, 1},  /* right_lower_elbow vs. left_hand */
    {22, 45, 303, 2},  /* right_lower_forearm vs. left_hand */
    {12, 45, 305, 1},  /* right_lower_shoulder vs. left_hand */
    {13, 45, 306, 3},  /* right_upper_elbow vs. left_hand */
    {18, 45, 309, 3},  /* right_upper_forearm vs. left_hand */
    {4, 45, 312, 2},  /* right_upper_shoulder vs. left_hand */
    {25, 45, 314, 2},  /* right_wrist vs. left_hand */
    {7, 45, 316, 3},  /* torso vs. left_hand */
    {11, 46, 319, 2},  /* head vs. left_gripper_base */
    {29, 46, 321, 2},  /* left_lower_shoulder vs. left_gripper_base */
    {30, 46, 323, 6},  /* left_upper_elbow vs. left_gripper_base */
    {0, 46, 329, 4},  /* left_upper_shoulder vs. left_gripper_base */
    {1, 46, 333, 2},  /* pedestal vs. left_gripper_base */
    {28, 46, 335, 2},  /* right_hand vs. left_gripper_base */
    {17, 46, 337, 2},  /* right_lower_elbow vs. left_gripper_base */
    {22, 46, 339, 4},  /* right_lower_forearm vs. left_gripper_base */
    {12, 46, 343, 2},  /* right_lower_shoulder vs. left_gripper_base */
    {13, 46, 345, 6},  /* right_upper_elbow vs. left_gripper_base */
    {18, 46, 351, 6},  /* right_upper_forearm vs. left_gripper_base */
    {4, 46, 357, 4},  /* right_upper_shoulder vs. left_gripper_base */
    {25, 46, 361, 4},  /* right_wrist vs. left_gripper_base */
    {7, 46, 365, 6},  /* torso vs. left_gripper_base */
    {29, 49, 371, 2},  /* left_lower_shoulder vs. l_gripper_l_finger */
    {30, 49, 373, 6},  /* left_upper_elbow vs. l_gripper_l_finger */
    {0, 49, 379, 4},  /* left_upper_shoulder vs. l_gripper_l_finger */
    {1, 49, 383, 2},  /* pedestal vs. l_gripper_l_finger */
    {28, 49, 385, 2},  /* right_hand vs. l_gripper_l_finger */
    {17, 49, 387, 2},  /* right_lower_elbow vs. l_gripper_l_finger */
    {22, 49, 389, 4},  /* right_lower_forearm vs. l_gripper_l_finger */
    {12, 49, 393, 2},  /* right_lower_shoulder vs. l_gripper_l_finger */
    {13, 49, 395, 6},  /* right_upper_elbow vs. l_gripper_l_finger */
    {18, 49, 401, 6},  /* right_upper_forearm vs. l_gripper_l_finger */
    {4, 49, 407, 4},  /* right_upper_shoulder vs. l_gripper_l_finger */
    {25, 49, 411, 4},  /* right_wrist vs. l_gripper_l_finger */
    {7, 49, 415, 6},  /* torso vs. l_gripper_l_finger */
    {29, 52, 421, 3},  /* left_lower_shoulder vs. l_gripper_l_finger_2 */
    {30, 52, 424, 9},  /* left_upper_elbow vs. l_gripper_l_finger_2 */
    {0, 52, 433, 6},  /* left_upper_shoulder vs. l_gripper_l_finger_2 */
    {1, 52, 439, 3},  /* pedestal vs. l_gripper_l_finger_2 */
    {28, 52, 442, 3},  /* right_hand vs. l_gripper_l_finger_2 */
    {17, 52, 445, 3},  /* right_lower_elbow vs. l_gripper_l_finger_2 */
    {22, 52, 448, 6},  /* right_lower_forearm vs. l_gripper_l_finger_2 */
    {12, 52, 454, 3},  /* right_lower_shoulder vs. l_gripper_l_finger_2 */
    {13, 52, 457, 9},  /* right_upper_elbow vs. l_gripper_l_finger_2 */
    {18, 52, 466, 9},  /* right_upper_forearm vs. l_gripper_l_finger_2 */
    {4, 52, 475, 6},  /* right_upper_shoulder vs. l_gripper_l_finger_2 */
    {25, 52, 481, 6},  /* right_wrist vs. l_gripper_l_finger_2 */
    {7, 52, 487, 9},  /* torso vs. l_gripper_l_finger_2 */
    {11, 56, 496, 4},  /* head vs. l_gripper_l_finger_tip */
    {34, 56, 500, 4},  /* left_lower_elbow vs. l_gripper_l_finger_tip */
    {29, 56, 504, 4},  /* left_lower_shoulder vs. l_gripper_l_finger_tip */
    {30, 56, 508, 12},  /* left_upper_elbow vs. l_gripper_l_finger_tip */
    {35, 56, 520, 12},  /* left_upper_forearm vs. l_gripper_l_finger_tip */
    {0, 56, 532, 8},  /* left_upper_shoulder vs. l_gripper_l_finger_tip */
    {1, 56, 540, 4},  /* pedestal vs. l_gripper_l_finger_tip */
    {28, 56, 544, 4},  /* right_hand vs. l_gripper_l_finger_tip */
    {17, 56, 548, 4},  /* right_lower_elbow vs. l_gripper_l_finger_tip */
    {22, 56, 552, 8},  /* right_lower_forearm vs. l_gripper_l_finger_tip */
    {12, 56, 560, 4},  /* right_lower_shoulder vs. l_gripper_l_finger_tip */
    {13, 56, 564, 12},  /* right_upper_elbow vs. l_gripper_l_finger_tip */
    {18, 56, 576, 12},  /* right_upper_forearm vs. l_gripper_l_finger_tip */
    {4, 56, 588, 8},  /* right_upper_shoulder vs. l_gripper_l_finger_tip */
    {25, 56, 596, 8},  /* right_wrist vs. l_gripper_l_finger_tip */
    {7, 56, 604, 12},  /* torso vs. l_gripper_l_finger_tip */
    {11, 61, 616, 2},  /* head vs. l_gripper_r_finger */
    {56, 61, 618, 8},  /* l_gripper_l_finger_tip vs. l_gripper_r_finger */
    {29, 61, 626, 2},  /* left_lower_shoulder vs. l_gripper_r_finger */
    {30, 61, 628, 6},  /* left_upper_elbow vs. l_gripper_r_finger */
    {0, 61, 634, 4},  /* left_upper_shoulder vs. l_gripper_r_finger */
    {1, 61, 638, 2},  /* pedestal vs. l_gripper_r_finger */
    {28, 61, 640, 2},  /* right_hand vs. l_gripper_r_finger */
    {17, 61, 642, 2},  /* right_lower_elbow vs. l_gripper_r_finger */
    {22, 61, 644, 4},  /* right_lower_forearm vs. l_gripper_r_finger */
    {12, 61, 648, 2},  /* right_lower_shoulder vs. l_gripper_r_finger */
    {13, 61, 650, 6},  /* right_upper_elbow vs. l_gripper_r_finger */
    {18, 61, 656, 6},  /* right_upper_forearm vs. l_gripper_r_finger */
    {4, 61, 662, 4},  /* right_upper_shoulder vs. l_gripper_r_finger */
    {25, 61, 666, 4},  /* right_wrist vs. l_gripper_r_finger */
    {7, 61, 670, 6},  /* torso vs. l_gripper_r_finger */
    {11, 64, 676, 3},  /* head vs. l_gripper_r_finger_2 */
    {56, 64, 679, 12},  /* l_gripper_l_finger_tip vs. l_gripper_r_finger_2 */
    {29, 64, 691, 3},  /* left_lower_shoulder vs. l_gripper_r_finger_2 */
    {30, 64, 694, 9},  /* left_upper_elbow vs. l_gripper_r_finger_2 */
    {0, 64, 703, 6},  /* left_upper_shoulder vs. l_gripper_r_finger_2 */
    {1, 64, 709, 3},  /* pedestal vs. l_gripper_r_finger_2 */
    {28, 64, 712, 3},  /* right_hand vs. l_gripper_r_finger_2 */
    {17, 64, 715, 3},  /* right_lower_elbow vs. l_gripper_r_finger_2 */
    {22, 64, 718, 6},  /* right_lower_forearm vs. l_gripper_r_finger_2 */
    {12, 64, 724, 3},  /* right_lower_shoulder vs. l_gripper_r_finger_2 */
    {13, 64, 727, 9},  /* right_upper_elbow vs. l_gripper_r_finger_2 */
    {18, 64, 736, 9},  /* right_upper_forearm vs. l_gripper_r_finger_2 */
    {4, 64, 745, 6},  /* right_upper_shoulder vs. l_gripper_r_finger_2 */
    {25, 64, 751, 6},  /* right_wrist vs. l_gripper_r_finger_2 */
    {7, 64, 757, 9},  /* torso vs. l_gripper_r_finger_2 */
    {11, 68, 766, 4},  /* head vs. l_gripper_r_finger_tip */
    {49, 68, 770, 8},  /* l_gripper_l_finger vs. l_gripper_r_finger_tip */
    {52, 68, 778, 12},  /* l_gripper_l_finger_2 vs. l_gripper_r_finger_tip */
    {56, 68, 790, 16},  /* l_gripper_l_finger_tip vs. l_gripper_r_finger_tip */
    {34, 68, 806, 4},  /* left_lower_elbow vs. l_gripper_r_finger_tip */
    {29, 68, 810, 4},  /* left_lower_shoulder vs. l_gripper_r_finger_tip */
    {30, 68, 814, 12},  /* left_upper_elbow vs. l_gripper_r_finger_tip */
    {35, 68, 826, 12},  /* left_upper_forearm vs. l_gripper_r_finger_tip */
    {0, 68, 838, 8},  /* left_upper_shoulder vs. l_gripper_r_finger_tip */
    {1, 68, 846, 4},  /* pedestal vs. l_gripper_r_finger_tip */
    {28, 68, 850, 4},  /* right_hand vs. l_gripper_r_finger_tip */
    {17, 68, 854, 4},  /* right_lower_elbow vs. l_gripper_r_finger_tip */
    {22, 68, 858, 8},  /* right_lower_forearm vs. l_gripper_r_finger_tip */
    {12, 68, 866, 4},  /* right_lower_shoulder vs. l_gripper_r_finger_tip */
    {13, 68, 870, 12},  /* right_upper_elbow vs. l_gripper_r_finger_tip */
    {18, 68, 882, 12},  /* right_upper_forearm vs. l_gripper_r_finger_tip */
    {4, 68, 894, 8},  /* right_upper_shoulder vs. l_gripper_r_finger_tip */
    {25, 68, 902, 8},  /* right_wrist vs. l_gripper_r_finger_tip */
    {7, 68, 910, 12},  /* torso vs. l_gripper_r_finger_tip */
    {11, 73, 922, 2},  /* head vs. right_gripper_base */
    {49, 73, 924, 4},  /* l_gripper_l_finger vs. right_gripper_base */
    {52, 73, 928, 6},  /* l_gripper_l_finger_2 vs. right_gripper_base */
    {56, 73, 934, 8},  /* l_gripper_l_finger_tip vs. right_gripper_base */
    {61, 73, 942, 4},  /* l_gripper_r_finger vs. right_gripper_base */
    {64, 73, 946, 6},  /* l_gripper_r_finger_2 vs. right_gripper_base */
    {68, 73, 952, 8},  /* l_gripper_r_finger_tip vs. right_gripper_base */
    {46, 73, 960, 4},  /* left_gripper_base vs. right_gripper_base */
    {45, 73, 964, 2},  /* left_hand vs. right_gripper_base */
    {34, 73, 966, 2},  /* left_lower_elbow vs. right_gripper_base */
    {39, 73, 968, 4},  /* left_lower_forearm vs. right_gripper_base */
    {29, 73, 972, 2},  /* left_lower_shoulder vs. right_gripper_base */
    {30, 73, 974, 6},  /* left_upper_elbow vs. right_gripper_base */
    {35, 73, 980, 6},  /* left_upper_forearm vs. right_gripper_base */
    {0, 73, 986, 4},  /* left_upper_shoulder vs. right_gripper_base */
    {42, 73, 990, 4},  /* left_wrist vs. right_gripper_base */
    {1, 73, 994, 2},  /* pedestal vs. right_gripper_base */
    {12, 73, 996, 2},  /* right_lower_shoulder vs. right_gripper_base */
    {13, 73, 998, 6},  /* right_upper_elbow vs. right_gripper_base */
    {4, 73, 1004, 4},  /* right_upper_shoulder vs. right_gripper_base */
    {7, 73, 1008, 6},  /* torso vs. right_gripper_base */
    {49, 76, 1014, 4},  /* l_gripper_l_finger vs. r_gripper_l_finger */
    {52, 76, 1018, 6},  /* l_gripper_l_finger_2 vs. r_gripper_l_finger */
    {56, 76, 1024, 8},  /* l_gripper_l_finger_tip vs. r_gripper_l_finger */
    {61, 76, 1032, 4},  /* l_gripper_r_finger vs. r_gripper_l_finger */
    {64, 76, 1036, 6},  /* l_gripper_r_finger_2 vs. r_gripper_l_finger */
    {68, 76, 1042, 8},  /* l_gripper_r_finger_tip vs. r_gripper_l_finger */
    {46, 76, 1050, 4},  /* left_gripper_base vs. r_gripper_l_finger */
    {45, 76, 1054, 2},  /* left_hand vs. r_gripper_l_finger */
    {34, 76, 1056, 2},  /* left_lower_elbow vs. r_gripper_l_finger */
    {39, 76, 1058, 4},  /* left_lower_forearm vs. r_gripper_l_finger */
    {29, 76, 1062, 2},  /* left_lower_shoulder vs. r_gripper_l_finger */
    {30, 76, 1064, 6},  /* left_upper_elbow vs. r_gripper_l_finger */
    {35, 76, 1070, 6},  /* left_upper_forearm vs. r_gripper_l_finger */
    {0, 76, 1076, 4},  /* left_upper_shoulder vs. r_gripper_l_finger */
    {42, 76, 1080, 4},  /* left_wrist vs. r_gripper_l_finger */
    {1, 76, 1084, 2},  /* pedestal vs. r_gripper_l_finger */
    {12, 76, 1086, 2},  /* right_lower_shoulder vs. r_gripper_l_finger */
    {13, 76, 1088, 6},  /* right_upper_elbow vs. r_gripper_l_finger */
    {4, 76, 1094, 4},  /* right_upper_shoulder vs. r_gripper_l_finger */
    {7, 76, 1098, 6},  /* torso vs. r_gripper_l_finger */
    {49, 79, 1104, 6},  /* l_gripper_l_finger vs. r_gripper_l_finger_2 */
    {52, 79, 1110, 9},  /* l_gripper_l_finger_2 vs. r_gripper_l_finger_2 */
    {56, 79, 1119, 12},  /* l_gripper_l_finger_tip vs. r_gripper_l_finger_2 */
    {61, 79, 1131, 6},  /* l_gripper_r_finger vs. r_gripper_l_finger_2 */
    {64, 79, 1137, 9},  /* l_gripper_r_finger_2 vs. r_gripper_l_finger_2 */
    {68, 79, 1146, 12},  /* l_gripper_r_finger_tip vs. r_gripper_l_finger_2 */
    {46, 79, 1158, 6},  /* left_gripper_base vs. r_gripper_l_finger_2 */
    {45, 79, 1164, 3},  /* left_hand vs. r_gripper_l_finger_2 */
    {34, 79, 1167, 3},  /* left_lower_elbow vs. r_gripper_l_finger_2 */
    {39, 79, 1170, 6},  /* left_lower_forearm vs. r_gripper_l_finger_2 */
    {29, 79, 1176, 3},  /* left_lower_shoulder vs. r_gripper_l_finger_2 */
    {30, 79, 1179, 9},  /* left_upper_elbow vs. r_gripper_l_finger_2 */
    {35, 79, 1188, 9},  /* left_upper_forearm vs. r_gripper_l_finger_2 */
    {0, 79, 1197, 6},  /* left_upper_shoulder vs. r_gripper_l_finger_2 */
    {42, 79, 1203, 6},  /* left_wrist vs. r_gripper_l_finger_2 */
    {1, 79, 1209, 3},  /* pedestal vs. r_gripper_l_finger_2 */
    {12, 79, 1212, 3},  /* right_lower_shoulder vs. r_gripper_l_finger_2 */
    {13, 79, 1215, 9},  /* right_upper_elbow vs. r_gripper_l_finger_2 */
    {4, 79, 1224, 6},  /* right_upper_shoulder vs. r_gripper_l_finger_2 */
    {7, 79, 1230, 9},  /* torso vs. r_gripper_l_finger_2 */
    {11, 83, 1239, 4},  /* head vs. r_gripper_l_finger_tip */
    {49, 83, 1243, 8},  /* l_gripper_l_finger vs. r_gripper_l_finger_tip */
    {52, 83, 1251, 12},  /* l_gripper_l_finger_2 vs. r_gripper_l_finger_tip */
    {56, 83, 1263, 16},  /* l_gripper_l_finger_tip vs. r_gripper_l_finger_tip */
    {61, 83, 1279, 8},  /* l_gripper_r_finger vs. r_gripper_l_finger_tip */
    {64, 83, 1287, 12},  /* l_gripper_r_finger_2 vs. r_gripper_l_finger_tip */
    {68, 83, 1299, 16},  /* l_gripper_r_finger_tip vs. r_gripper_l_finger_tip */
    {46, 83, 1315, 8},  /* left_gripper_base vs. r_gripper_l_finger_tip */
    {45, 83, 1323, 4},  /* left_hand vs. r_gripper_l_finger_tip */
    {34, 83, 1327, 4},  /* left_lower_elbow vs. r_gripper_l_finger_tip */
    {39, 83, 1331, 8},  /* left_lower_forearm vs. r_gripper_l_finger_tip */
    {29, 83, 1339, 4},  /* left_lower_shoulder vs. r_gripper_l_finger_tip */
    {30, 83, 1343, 12},  /* left_upper_elbow vs. r_gripper_l_finger_tip */
    {35, 83, 1355, 12},  /* left_upper_forearm vs. r_gripper_l_finger_tip */
    {0, 83, 1367, 8},  /* left_upper_shoulder vs. r_gripper_l_finger_tip */
    {42, 83, 1375, 8},  /* left_wrist vs. r_gripper_l_finger_tip */
    {1, 83, 1383, 4},  /* pedestal vs. r_gripper_l_finger_tip */
    {17, 83, 1387, 4},  /* right_lower_elbow vs. r_gripper_l_finger_tip */
    {12, 83, 1391, 4},  /* right_lower_shoulder vs. r_gripper_l_finger_tip */
    {13, 83, 1395, 12},  /* right_upper_elbow vs. r_gripper_l_finger_tip */
    {18, 83, 1407, 12},  /* right_upper_forearm vs. r_gripper_l_finger_tip */
    {4, 83, 1419, 8},  /* right_upper_shoulder vs. r_gripper_l_finger_tip */
    {7, 83, 1427, 12},  /* torso vs. r_gripper_l_finger_tip */
    {11, 88, 1439, 2},  /* head vs. r_gripper_r_finger */
    {49, 88, 1441, 4},  /* l_gripper_l_finger vs. r_gripper_r_finger */
    {52, 88, 1445, 6},  /* l_gripper_l_finger_2 vs. r_gripper_r_finger */
    {56, 88, 1451, 8},  /* l_gripper_l_finger_tip vs. r_gripper_r_finger */
    {61, 88, 1459, 4},  /* l_gripper_r_finger vs. r_gripper_r_finger */
    {64, 88, 1463, 6},  /* l_gripper_r_finger_2 vs. r_gripper_r_finger */
    {68, 88, 1469, 8},  /* l_gripper_r_finger_tip vs. r_gripper_r_finger */
    {46, 88, 1477, 4},  /* left_gripper_base vs. r_gripper_r_finger */
    {45, 88, 1481, 2},  /* left_hand vs. r_gripper_r_finger */
    {34, 88, 1483, 2},  /* left_lower_elbow vs. r_gripper_r_finger */
    {39, 88, 1485, 4},  /* left_lower_forearm vs. r_gripper_r_finger */
    {29, 88, 1489, 2},  /* left_lower_shoulder vs. r_gripper_r_finger */
    {30, 88, 1491, 6},  /* left_upper_elbow vs. r_gripper_r_finger */
    {35, 88, 1497, 6},  /* left_upper_forearm vs. r_gripper_r_finger */
    {0, 88, 1503, 4},  /* left_upper_shoulder vs. r_gripper_r_finger */
    {42, 88, 1507, 4},  /* left_wrist vs. r_gripper_r_finger */
    {1, 88, 1511, 2},  /* pedestal vs. r_gripper_r_finger */
    {83, 88, 1513, 8},  /* r_gripper_l_finger_tip vs. r_gripper_r_finger */
    {12, 88, 1521, 2},  /* right_lower_shoulder vs. r_gripper_r_finger */
    {13, 88, 1523, 6},  /* right_upper_elbow vs. r_gripper_r_finger */
    {4, 88, 1529, 4},  /* right_upper_shoulder vs. r_gripper_r_finger */
    {7, 88, 1533, 6},  /* torso vs. r_gripper_r_finger */
    {11, 91, 1539, 3},  /* head vs. r_gripper_r_finger_2 */
    {49, 91, 1542, 6},  /* l_gripper_l_finger vs. r_gripper_r_finger_2 */
    {52, 91, 1548, 9},  /* l_gripper_l_finger_2 vs. r_gripper_r_finger_2 */
    {56, 91, 1557, 12},  /* l_gripper_l_finger_tip vs. r_gripper_r_finger_2 */
    {61, 91, 1569, 6},  /* l_gripper_r_finger vs. r_gripper_r_finger_2 */
    {64, 91, 1575, 9},  /* l_gripper_r_finger_2 vs. r_gripper_r_finger_2 */
    {68, 91, 1584, 12},  /* l_gripper_r_finger_tip vs. r_gripper_r_finger_2 */
    {46, 91, 1596, 6},  /* left_gripper_base vs. r_gripper_r_finger_2 */
    {45, 91, 1602, 3},  /* left_hand vs. r_gripper_r_finger_2 */
    {34, 91, 1605, 3},  /* left_lower_elbow vs. r_gripper_r_finger_2 */
    {39, 91, 1608, 6},  /* left_lower_forearm vs. r_gripper_r_finger_2 */
    {29, 91, 1614, 3},  /* left_lower_shoulder vs. r_gripper_r_finger_2 */
    {30, 91, 1617, 9},  /* left_upper_elbow vs. r_gripper_r_finger_2 */
    {35, 91, 1626, 9},  /* left_upper_forearm vs. r_gripper_r_finger_2 */
    {0, 91, 1635, 6},  /* left_upper_shoulder vs. r_gripper_r_finger_2 */
    {42, 91, 1641, 6},  /* left_wrist vs. r_gripper_r_finger_2 */
    {1, 91, 1647, 3},  /* pedestal vs. r_gripper_r_finger_2 */
    {83, 91, 1650, 12},  /* r_gripper_l_finger_tip vs. r_gripper_r_finger_2 */
    {12, 91, 1662, 3},  /* right_lower_shoulder vs. r_gripper_r_finger_2 */
    {13, 91, 1665, 9},  /* right_upper_elbow vs. r_gripper_r_finger_2 */
    {4, 91, 1674, 6},  /* right_upper_shoulder vs. r_gripper_r_finger_2 */
    {7, 91, 1680, 9},  /* torso vs. r_gripper_r_finger_2 */
    {11, 95, 1689, 4},  /* head vs. r_gripper_r_finger_tip */
    {49, 95, 1693, 8},  /* l_gripper_l_finger vs. r_gripper_r_finger_tip */
    {52, 95, 1701, 12},  /* l_gripper_l_finger_2 vs. r_gripper_r_finger_tip */
    {56, 95, 1713, 16},  /* l_gripper_l_finger_tip vs. r_gripper_r_finger_tip */
    {61, 95, 1729, 8},  /* l_gripper_r_finger vs. r_gripper_r_finger_tip */
    {64, 95, 1737, 12},  /* l_gripper_r_finger_2 vs. r_gripper_r_finger_tip */
    {68, 95, 1749, 16},  /* l_gripper_r_finger_tip vs. r_gripper_r_finger_tip */
    {46, 95, 1765, 8},  /* left_gripper_base vs. r_gripper_r_finger_tip */
    {45, 95, 1773, 4},  /* left_hand vs. r_gripper_r_finger_tip */
    {34, 95, 1777, 4},  /* left_lower_elbow vs. r_gripper_r_finger_tip */
    {39, 95, 1781, 8},  /* left_lower_forearm vs. r_gripper_r_finger_tip */
    {29, 95, 1789, 4},  /* left_lower_shoulder vs. r_gripper_r_finger_tip */
    {30, 95, 1793, 12},  /* left_upper_elbow vs. r_gripper_r_finger_tip */
    {35, 95, 1805, 12},  /* left_upper_forearm vs. r_gripper_r_finger_tip */
    {0, 95, 1817, 8},  /* left_upper_shoulder vs. r_gripper_r_finger_tip */
    {42, 95, 1825, 8},  /* left_wrist vs. r_gripper_r_finger_tip */
    {1, 95, 1833, 4},  /* pedestal vs. r_gripper_r_finger_tip */
    {76, 95, 1837, 8},  /* r_gripper_l_finger vs. r_gripper_r_finger_tip */
    {79, 95, 1845, 12},  /* r_gripper_l_finger_2 vs. r_gripper_r_finger_tip */
    {83, 95, 1857, 16},  /* r_gripper_l_finger_tip vs. r_gripper_r_finger_tip */
    {17, 95, 1873, 4},  /* right_lower_elbow vs. r_gripper_r_finger_tip */
    {12, 95, 1877, 4},  /* right_lower_shoulder vs. r_gripper_r_finger_tip */
    {13, 95, 1881, 12},  /* right_upper_elbow vs. r_gripper_r_finger_tip */
    {18, 95, 1893, 12},  /* right_upper_forearm vs. r_gripper_r_finger_tip */
    {4, 95, 1905, 8},  /* right_upper_shoulder vs. r_gripper_r_finger_tip */
    {7, 95, 1913, 12},  /* torso vs. r_gripper_r_finger_tip */
};
static const short kBaxterSelfPairs[][2] = {
    {2, 1}, {3, 1}, {11, 17}, {8, 17}, {9, 17}, {10, 17}, {11, 19}, {11, 20},
    {11, 21}, {19, 1}, {20, 1}, {21, 1}, {5, 19}, {5, 20}, {5, 21}, {6, 19},
    {6, 20}, {6, 21}, {8, 19}, {8, 20}, {8, 21}, {9, 19}, {9, 20}, {9, 21},
    {10, 19}, {10, 20}, {10, 21}, {11, 23}, {11, 24}, {23, 2}, {23, 3}, {24, 2},
    {24, 3}, {23, 1}, {24, 1}, {5, 23}, {5, 24}, {6, 23}, {6, 24}, {8, 23},
    {8, 24}, {9, 23}, {9, 24}, {10, 23}, {10, 24}, {11, 26}, {11, 27}, {12, 26},
    {12, 27}, {14, 26}, {14, 27}, {15, 26}, {15, 27}, {16, 26}, {16, 27}, {5, 26},
    {5, 27}, {6, 26}, {6, 27}, {26, 2}, {26, 3}, {27, 2}, {27, 3}, {26, 1},
    {27, 1}, {8, 26}, {8, 27}, {9, 26}, {9, 27}, {10, 26}, {10, 27}, {11, 28},
    {28, 2}, {28, 3}, {28, 1}, {12, 28}, {14, 28}, {15, 28}, {16, 28}, {5, 28},
    {6, 28}, {8, 28}, {9, 28}, {10, 28}, {28, 29}, {17, 29}, {23, 29}, {24, 29},
    {19, 29}, {20, 29}, {21, 29}, {26, 29}, {27, 29}, {28, 31}, {28, 32}, {28, 33},
    {17, 31}, {17, 32}, {17, 33}, {23, 31}, {23, 32}, {23, 33}, {24, 31}, {24, 32},
    {24, 33}, {19, 31}, {19, 32}, {19, 33}, {20, 31}, {20, 32}, {20, 33}, {21, 31},
    {21, 32}, {21, 33}, {26, 31}, {26, 32}, {26, 33}, {27, 31}, {27, 32}, {27, 33},
    {11, 34}, {28, 34}, {17, 34}, {23, 34}, {24, 34}, {12, 34}, {14, 34}, {15, 34},
    {16, 34}, {19, 34}, {20, 34}, {21, 34}, {26, 34}, {27, 34}, {8, 34}, {9, 34},
    {10, 34}, {11, 36}, {11, 37}, {11, 38}, {36, 1}, {37, 1}, {38, 1}, {2, 36},
    {2, 37}, {2, 38}, {3, 36}, {3, 37}, {3, 38}, {28, 36}, {28, 37}, {28, 38},
    {17, 36}, {17, 37}, {17, 38}, {23, 36}, {23, 37}, {23, 38}, {24, 36}, {24, 37},
    {24, 38}, {12, 36}, {12, 37}, {12, 38}, {14, 36}, {14, 37}, {14, 38}, {15, 36},
    {15, 37}, {15, 38}, {16, 36}, {16, 37}, {16, 38}, {19, 36}, {19, 37}, {19, 38},
    {20, 36}, {20, 37}, {20, 38}, {21, 36}, {21, 37}, {21, 38}, {26, 36}, {26, 37},
    {26, 38}, {27, 36}, {27, 37}, {27, 38}, {8, 36}, {8, 37}, {8, 38}, {9, 36},
    {9, 37}, {9, 38}, {10, 36}, {10, 37}, {10, 38}, {11, 40}, {11, 41}, {40, 1},
    {41, 1}, {2, 40}, {2, 41}, {3, 40}, {3, 41}, {28, 40}, {28, 41}, {17, 40},
    {17, 41}, {23, 40}, {23, 41}, {24, 40}, {24, 41}, {12, 40}, {12, 41}, {14, 40},
    {14, 41}, {15, 40}, {15, 41}, {16, 40}, {16, 41}, {19, 40}, {19, 41}, {20, 40},
    {20, 41}, {21, 40}, {21, 41}, {5, 40}, {5, 41}, {6, 40}, {6, 41}, {26, 40},
    {26, 41}, {27, 40}, {27, 41}, {8, 40}, {8, 41}, {9, 40}, {9, 41}, {10, 40},
    {10, 41}, {11, 43}, {11, 44}, {29, 43}, {29, 44}, {31, 43}, {31, 44}, {32, 43},
    {32, 44}, {33, 43}, {33, 44}, {2, 43}, {2, 44}, {3, 43}, {3, 44}, {43, 1},
    {44, 1}, {28, 43}, {28, 44}, {17, 43}, {17, 44}, {23, 43}, {23, 44}, {24, 43},
    {24, 44}, {12, 43}, {12, 44}, {14, 43}, {14, 44}, {15, 43}, {15, 44}, {16, 43},
    {16, 44}, {19, 43}, {19, 44}, {20, 43}, {20, 44}, {21, 43}, {21, 44}, {5, 43},
    {5, 44}, {6, 43}, {6, 44}, {26, 43}, {26, 44}, {27, 43}, {27, 44}, {8, 43},
    {8, 44}, {9, 43}, {9, 44}, {10, 43}, {10, 44}, {11, 45}, {45, 1}, {29, 45},
    {31, 45}, {32, 45}, {33, 45}, {2, 45}, {3, 45}, {28, 45}, {17, 45}, {23, 45},
    {24, 45}, {12, 45}, {14, 45}, {15, 45}, {16, 45}, {19, 45}, {20, 45}, {21, 45},
    {5, 45}, {6, 45}, {26, 45}, {27, 45}, {8, 45}, {9, 45}, {10, 45}, {11, 47},
    {11, 48}, {29, 47}, {29, 48}, {31, 47}, {31, 48}, {32, 47}, {32, 48}, {33, 47},
    {33, 48}, {2, 47}, {2, 48}, {3, 47}, {3, 48}, {1, 47}, {1, 48}, {28, 47},
    {28, 48}, {17, 47}, {17, 48}, {23, 47}, {23, 48}, {24, 47}, {24, 48}, {12, 47},
    {12, 48}, {14, 47}, {14, 48}, {15, 47}, {15, 48}, {16, 47}, {16, 48}, {19, 47},
    {19, 48}, {20, 47}, {20, 48}, {21, 47}, {21, 48}, {5, 47}, {5, 48}, {6, 47},
    {6, 48}, {26, 47}, {26, 48}, {27, 47}, {27, 48}, {8, 47}, {8, 48}, {9, 47},
    {9, 48}, {10, 47}, {10, 48}, {29, 50}, {29, 51}, {31, 50}, {31, 51}, {32, 50},
    {32, 51}, {33, 50}, {33, 51}, {2, 50}, {2, 51}, {3, 50}, {3, 51}, {1, 50},
    {1, 51}, {28, 50}, {28, 51}, {17, 50}, {17, 51}, {23, 50}, {23, 51}, {24, 50},
    {24, 51}, {12, 50}, {12, 51}, {14, 50}, {14, 51}, {15, 50}, {15, 51}, {16, 50},
    {16, 51}, {19, 50}, {19, 51}, {20, 50}, {20, 51}, {21, 50}, {21, 51}, {5, 50},
    {5, 51}, {6, 50}, {6, 51}, {26, 50}, {26, 51}, {27, 50}, {27, 51}, {8, 50},
    {8, 51}, {9, 50}, {9, 51}, {10, 50}, {10, 51}, {29, 53}, {29, 54}, {29, 55},
    {31, 53}, {31, 54}, {31, 55}, {32, 53}, {32, 54}, {32, 55}, {33, 53}, {33, 54},
    {33, 55}, {2, 53}, {2, 54}, {2, 55}, {3, 53}, {3, 54}, {3, 55}, {1, 53},
    {1, 54}, {1, 55}, {28, 53}, {28, 54}, {28, 55}, {17, 53}, {17, 54}, {17, 55},
    {23, 53}, {23, 54}, {23, 55}, {24, 53}, {24, 54}, {24, 55}, {12, 53}, {12, 54},
    {12, 55}, {14, 53}, {14, 54}, {14, 55}, {15, 53}, {15, 54}, {15, 55}, {16, 53},
    {16, 54}, {16, 55}, {19, 53}, {19, 54}, {19, 55}, {20, 53}, {20, 54}, {20, 55},
    {21, 53}, {21, 54}, {21, 55}, {5, 53}, {5, 54}, {5, 55}, {6, 53}, {6, 54},
    {6, 55}, {26, 53}, {26, 54}, {26, 55}, {27, 53}, {27, 54}, {27, 55}, {8, 53},
    {8, 54}, {8, 55}, {9, 53}, {9, 54}, {9, 55}, {10, 53}, {10, 54}, {10, 55},
    {11, 57}, {11, 58}, {11, 59}, {11, 60}, {34, 57}, {34, 58}, {34, 59}, {34, 60},
    {29, 57}, {29, 58}, {29, 59}, {29, 60}, {31, 57}, {31, 58}, {31, 59}, {31, 60},
    {32, 57}, {32, 58}, {32, 59}, {32, 60}, {33, 57}, {33, 58}, {33, 59}, {33, 60},
    {36, 57}, {36, 58}, {36, 59}, {36, 60}, {37, 57}, {37, 58}, {37, 59}, {37, 60},
    {38, 57}, {38, 58}, {38, 59}, {38, 60}, {2, 57}, {2, 58}, {2, 59}, {2, 60},
    {3, 57}, {3, 58}, {3, 59}, {3, 60}, {1, 57}, {1, 58}, {1, 59}, {1, 60},
    {28, 57}, {28, 58}, {28, 59}, {28, 60}, {17, 57}, {17, 58}, {17, 59}, {17, 60},
    {23, 57}, {23, 58}, {23, 59}, {23, 60}, {24, 57}, {24, 58}, {24, 59}, {24, 60},
    {12, 57}, {12, 58}, {12, 59}, {12, 60}, {14, 57}, {14, 58}, {14, 59}, {14, 60},
    {15, 57}, {15, 58}, {15, 59}, {15, 60}, {16, 57}, {16, 58}, {16, 59}, {16, 60},
    {19, 57}, {19, 58}, {19, 59}, {19, 60}, {20, 57}, {20, 58}, {20, 59}, {20, 60},
    {21, 57}, {21, 58}, {21, 59}, {21, 60}, {5, 57}, {5, 58}, {5, 59}, {5, 60},
    {6, 57}, {6, 58}, {6, 59}, {6, 60}, {26, 57}, {26, 58}, {26, 59}, {26, 60},
    {27, 57}, {27, 58}, {27, 59}, {27, 60}, {8, 57}, {8, 58}, {8, 59}, {8, 60},
    {9, 57}, {9, 58}, {9, 59}, {9, 60}, {10, 57}, {10, 58}, {10, 59}, {10, 60},
    {11, 62}, {11, 63}, {57, 62}, {57, 63}, {58, 62}, {58, 63}, {59, 62}, {59, 63},
    {60, 62}, {60, 63}, {29, 62}, {29, 63}, {31, 62}, {31, 63}, {32, 62}, {32, 63},
    {33, 62}, {33, 63}, {2, 62}, {2, 63}, {3, 62}, {3, 63}, {1, 62}, {1, 63},
    {28, 62}, {28, 63}, {17, 62}, {17, 63}, {23, 62}, {23, 63}, {24, 62}, {24, 63},
    {12, 62}, {12, 63}, {14, 62}, {14, 63}, {15, 62}, {15, 63}, {16, 62}, {16, 63},
    {19, 62}, {19, 63}, {20, 62}, {20, 63}, {21, 62}, {21, 63}, {5, 62}, {5, 63},
    {6, 62}, {6, 63}, {26, 62}, {26, 63}, {27, 62}, {27, 63}, {8, 62}, {8, 63},
    {9, 62}, {9, 63}, {10, 62}, {10, 63}, {11, 65}, {11, 66}, {11, 67}, {57, 65},
    {57, 66}, {57, 67}, {58, 65}, {58, 66}, {58, 67}, {59, 65}, {59, 66}, {59, 67},
    {60, 65}, {60, 66}, {60, 67}, {29, 65}, {29, 66}, {29, 67}, {31, 65}, {31, 66},
    {31, 67}, {32, 65}, {32, 66}, {32, 67}, {33, 65}, {33, 66}, {33, 67}, {2, 65},
    {2, 66}, {2, 67}, {3, 65}, {3, 66}, {3, 67}, {1, 65}, {1, 66}, {1, 67},
    {28, 65}, {28, 66}, {28, 67}, {17, 65}, {17, 66}, {17, 67}, {23, 65}, {23, 66},
    {23, 67}, {24, 65}, {24, 66}, {24, 67}, {12, 65}, {12, 66}, {12, 67}, {14, 65},
    {14, 66}, {14, 67}, {15, 65}, {15, 66}, {15, 67}, {16, 65}, {16, 66}, {16, 67},
    {19, 65}, {19, 66}, {19, 67}, {20, 65}, {20, 66}, {20, 67}, {21, 65}, {21, 66},
    {21, 67}, {5, 65}, {5, 66}, {5, 67}, {6, 65}, {6, 66}, {6, 67}, {26, 65},
    {26, 66}, {26, 67}, {27, 65}, {27, 66}, {27, 67}, {8, 65}, {8, 66}, {8, 67},
    {9, 65}, {9, 66}, {9, 67}, {10, 65}, {10, 66}, {10, 67}, {11, 69}, {11, 70},
    {11, 71}, {11, 72}, {50, 69}, {50, 70}, {50, 71}, {50, 72}, {51, 69}, {51, 70},
    {51, 71}, {51, 72}, {53, 69}, {53, 70}, {53, 71}, {53, 72}, {54, 69}, {54, 70},
    {54, 71}, {54, 72}, {55, 69}, {55, 70}, {55, 71}, {55, 72}, {57, 69}, {57, 70},
    {57, 71}, {57, 72}, {58, 69}, {58, 70}, {58, 71}, {58, 72}, {59, 69}, {59, 70},
    {59, 71}, {59, 72}, {60, 69}, {60, 70}, {60, 71}, {60, 72}, {34, 69}, {34, 70},
    {34, 71}, {34, 72}, {29, 69}, {29, 70}, {29, 71}, {29, 72}, {31, 69}, {31, 70},
    {31, 71}, {31, 72}, {32, 69}, {32, 70}, {32, 71}, {32, 72}, {33, 69}, {33, 70},
    {33, 71}, {33, 72}, {36, 69}, {36, 70}, {36, 71}, {36, 72}, {37, 69}, {37, 70},
    {37, 71}, {37, 72}, {38, 69}, {38, 70}, {38, 71}, {38, 72}, {2, 69}, {2, 70},
    {2, 71}, {2, 72}, {3, 69}, {3, 70}, {3, 71}, {3, 72}, {1, 69}, {1, 70},
    {1, 71}, {1, 72}, {28, 69}, {28, 70}, {28, 71}, {28, 72}, {17, 69}, {17, 70},
    {17, 71}, {17, 72}, {23, 69}, {23, 70}, {23, 71}, {23, 72}, {24, 69}, {24, 70},
    {24, 71}, {24, 72}, {12, 69}, {12, 70}, {12, 71}, {12, 72}, {14, 69}, {14, 70},
    {14, 71}, {14, 72}, {15, 69}, {15, 70}, {15, 71}, {15, 72}, {16, 69}, {16, 70},
    {16, 71}, {16, 72}, {19, 69}, {19, 70}, {19, 71}, {19, 72}, {20, 69}, {20, 70},
    {20, 71}, {20, 72}, {21, 69}, {21, 70}, {21, 71}, {21, 72}, {5, 69}, {5, 70},
    {5, 71}, {5, 72}, {6, 69}, {6, 70}, {6, 71}, {6, 72}, {26, 69}, {26, 70},
    {26, 71}, {26, 72}, {27, 69}, {27, 70}, {27, 71}, {27, 72}, {8, 69}, {8, 70},
    {8, 71}, {8, 72}, {9, 69}, {9, 70}, {9, 71}, {9, 72}, {10, 69}, {10, 70},
    {10, 71}, {10, 72}, {11, 74}, {11, 75}, {50, 74}, {50, 75}, {51, 74}, {51, 75},
    {53, 74}, {53, 75}, {54, 74}, {54, 75}, {55, 74}, {55, 75}, {57, 74}, {57, 75},
    {58, 74}, {58, 75}, {59, 74}, {59, 75}, {60, 74}, {60, 75}, {62, 74}, {62, 75},
    {63, 74}, {63, 75}, {65, 74}, {65, 75}, {66, 74}, {66, 75}, {67, 74}, {67, 75},
    {69, 74}, {69, 75}, {70, 74}, {70, 75}, {71, 74}, {71, 75}, {72, 74}, {72, 75},
    {47, 74}, {47, 75}, {48, 74}, {48, 75}, {45, 74}, {45, 75}, {34, 74}, {34, 75},
    {40, 74}, {40, 75}, {41, 74}, {41, 75}, {29, 74}, {29, 75}, {31, 74}, {31, 75},
    {32, 74}, {32, 75}, {33, 74}, {33, 75}, {36, 74}, {36, 75}, {37, 74}, {37, 75},
    {38, 74}, {38, 75}, {2, 74}, {2, 75}, {3, 74}, {3, 75}, {43, 74}, {43, 75},
    {44, 74}, {44, 75}, {1, 74}, {1, 75}, {12, 74}, {12, 75}, {14, 74}, {14, 75},
    {15, 74}, {15, 75}, {16, 74}, {16, 75}, {5, 74}, {5, 75}, {6, 74}, {6, 75},
    {8, 74}, {8, 75}, {9, 74}, {9, 75}, {10, 74}, {10, 75}, {50, 77}, {50, 78},
    {51, 77}, {51, 78}, {53, 77}, {53, 78}, {54, 77}, {54, 78}, {55, 77}, {55, 78},
    {57, 77}, {57, 78}, {58, 77}, {58, 78}, {59, 77}, {59, 78}, {60, 77}, {60, 78},
    {62, 77}, {62, 78}, {63, 77}, {63, 78}, {65, 77}, {65, 78}, {66, 77}, {66, 78},
    {67, 77}, {67, 78}, {69, 77}, {69, 78}, {70, 77}, {70, 78}, {71, 77}, {71, 78},
    {72, 77}, {72, 78}, {47, 77}, {47, 78}, {48, 77}, {48, 78}, {45, 77}, {45, 78},
    {34, 77}, {34, 78}, {40, 77}, {40, 78}, {41, 77}, {41, 78}, {29, 77}, {29, 78},
    {31, 77}, {31, 78}, {32, 77}, {32, 78}, {33, 77}, {33, 78}, {36, 77}, {36, 78},
    {37, 77}, {37, 78}, {38, 77}, {38, 78}, {2, 77}, {2, 78}, {3, 77}, {3, 78},
    {43, 77}, {43, 78}, {44, 77}, {44, 78}, {1, 77}, {1, 78}, {12, 77}, {12, 78},
    {14, 77}, {14, 78}, {15, 77}, {15, 78}, {16, 77}, {16, 78}, {5, 77}, {5, 78},
    {6, 77}, {6, 78}, {8, 77}, {8, 78}, {9, 77}, {9, 78}, {10, 77}, {10, 78},
    {50, 80}, {50, 81}, {50, 82}, {51, 80}, {51, 81}, {51, 82}, {53, 80}, {53, 81},
    {53, 82}, {54, 80}, {54, 81}, {54, 82}, {55, 80}, {55, 81}, {55, 82}, {57, 80},
    {57, 81}, {57, 82}, {58, 80}, {58, 81}, {58, 82}, {59, 80}, {59, 81}, {59, 82},
    {60, 80}, {60, 81}, {60, 82}, {62, 80}, {62, 81}, {62, 82}, {63, 80}, {63, 81},
    {63, 82}, {65, 80}, {65, 81}, {65, 82}, {66, 80}, {66, 81}, {66, 82}, {67, 80},
    {67, 81}, {67, 82}, {69, 80}, {69, 81}, {69, 82}, {70, 80}, {70, 81}, {70, 82},
    {71, 80}, {71, 81}, {71, 82}, {72, 80}, {72, 81}, {72, 82}, {47, 80}, {47, 81},
    {47, 82}, {48, 80}, {48, 81}, {48, 82}, {45, 80}, {45, 81}, {45, 82}, {34, 80},
    {34, 81}, {34, 82}, {40, 80}, {40, 81}, {40, 82}, {41, 80}, {41, 81}, {41, 82},
    {29, 80}, {29, 81}, {29, 82}, {31, 80}, {31, 81}, {31, 82}, {32, 80}, {32, 81},
    {32, 82}, {33, 80}, {33, 81}, {33, 82}, {36, 80}, {36, 81}, {36, 82}, {37, 80},
    {37, 81}, {37, 82}, {38, 80}, {38, 81}, {38, 82}, {2, 80}, {2, 81}, {2, 82},
    {3, 80}, {3, 81}, {3, 82}, {43, 80}, {43, 81}, {43, 82}, {44, 80}, {44, 81},
    {44, 82}, {1, 80}, {1, 81}, {1, 82}, {12, 80}, {12, 81}, {12, 82}, {14, 80},
    {14, 81}, {14, 82}, {15, 80}, {15, 81}, {15, 82}, {16, 80}, {16, 81}, {16, 82},
    {5, 80}, {5, 81}, {5, 82}, {6, 80}, {6, 81}, {6, 82}, {8, 80}, {8, 81},
    {8, 82}, {9, 80}, {9, 81}, {9, 82}, {10, 80}, {10, 81}, {10, 82}, {11, 84},
    {11, 85}, {11, 86}, {11, 87}, {50, 84}, {50, 85}, {50, 86}, {50, 87}, {51, 84},
    {51, 85}, {51, 86}, {51, 87}, {53, 84}, {53, 85}, {53, 86}, {53, 87}, {54, 84},
    {54, 85}, {54, 86}, {54, 87}, {55, 84}, {55, 85}, {55, 86}, {55, 87}, {57, 84},
    {57, 85}, {57, 86}, {57, 87}, {58, 84}, {58, 85}, {58, 86}, {58, 87}, {59, 84},
    {59, 85}, {59, 86}, {59, 87}, {60, 84}, {60, 85}, {60, 86}, {60, 87}, {62, 84},
    {62, 85}, {62, 86}, {62, 87}, {63, 84}, {63, 85}, {63, 86}, {63, 87}, {65, 84},
    {65, 85}, {65, 86}, {65, 87}, {66, 84}, {66, 85}, {66, 86}, {66, 87}, {67, 84},
    {67, 85}, {67, 86}, {67, 87}, {69, 84}, {69, 85}, {69, 86}, {69, 87}, {70, 84},
    {70, 85}, {70, 86}, {70, 87}, {71, 84}, {71, 85}, {71, 86}, {71, 87}, {72, 84},
    {72, 85}, {72, 86}, {72, 87}, {47, 84}, {47, 85}, {47, 86}, {47, 87}, {48, 84},
    {48, 85}, {48, 86}, {48, 87}, {45, 84}, {45, 85}, {45, 86}, {45, 87}, {34, 84},
    {34, 85}, {34, 86}, {34, 87}, {40, 84}, {40, 85}, {40, 86}, {40, 87}, {41, 84},
    {41, 85}, {41, 86}, {41, 87}, {29, 84}, {29, 85}, {29, 86}, {29, 87}, {31, 84},
    {31, 85}, {31, 86}, {31, 87}, {32, 84}, {32, 85}, {32, 86}, {32, 87}, {33, 84},
    {33, 85}, {33, 86}, {33, 87}, {36, 84}, {36, 85}, {36, 86}, {36, 87}, {37, 84},
    {37, 85}, {37, 86}, {37, 87}, {38, 84}, {38, 85}, {38, 86}, {38, 87}, {2, 84},
    {2, 85}, {2, 86}, {2, 87}, {3, 84}, {3, 85}, {3, 86}, {3, 87}, {43, 84},
    {43, 85}, {43, 86}, {43, 87}, {44, 84}, {44, 85}, {44, 86}, {44, 87}, {1, 84},
    {1, 85}, {1, 86}, {1, 87}, {17, 84}, {17, 85}, {17, 86}, {17, 87}, {12, 84},
    {12, 85}, {12, 86}, {12, 87}, {14, 84}, {14, 85}, {14, 86}, {14, 87}, {15, 84},
    {15, 85}, {15, 86}, {15, 87}, {16, 84}, {16, 85}, {16, 86}, {16, 87}, {19, 84},
    {19, 85}, {19, 86}, {19, 87}, {20, 84}, {20, 85}, {20, 86}, {20, 87}, {21, 84},
    {21, 85}, {21, 86}, {21, 87}, {5, 84}, {5, 85}, {5, 86}, {5, 87}, {6, 84},
    {6, 85}, {6, 86}, {6, 87}, {8, 84}, {8, 85}, {8, 86}, {8, 87}, {9, 84},
    {9, 85}, {9, 86}, {9, 87}, {10, 84}, {10, 85}, {10, 86}, {10, 87}, {11, 89},
    {11, 90}, {50, 89}, {50, 90}, {51, 89}, {51, 90}, {53, 89}, {53, 90}, {54, 89},
    {54, 90}, {55, 89}, {55, 90}, {57, 89}, {57, 90}, {58, 89}, {58, 90}, {59, 89},
    {59, 90}, {60, 89}, {60, 90}, {62, 89}, {62, 90}, {63, 89}, {63, 90}, {65, 89},
    {65, 90}, {66, 89}, {66, 90}, {67, 89}, {67, 90}, {69, 89}, {69, 90}, {70, 89},
    {70, 90}, {71, 89}, {71, 90}, {72, 89}, {72, 90}, {47, 89}, {47, 90}, {48, 89},
    {48, 90}, {45, 89}, {45, 90}, {34, 89}, {34, 90}, {40, 89}, {40, 90}, {41, 89},
    {41, 90}, {29, 89}, {29, 90}, {31, 89}, {31, 90}, {32, 89}, {32, 90}, {33, 89},
    {33, 90}, {36, 89}, {36, 90}, {37, 89}, {37, 90}, {38, 89}, {38, 90}, {2, 89},
    {2, 90}, {3, 89}, {3, 90}, {43, 89}, {43, 90}, {44, 89}, {44, 90}, {1, 89},
    {1, 90}, {84, 89}, {84, 90}, {85, 89}, {85, 90}, {86, 89}, {86, 90}, {87, 89},
    {87, 90}, {12, 89}, {12, 90}, {14, 89}, {14, 90}, {15, 89}, {15, 90}, {16, 89},
    {16, 90}, {5, 89}, {5, 90}, {6, 89}, {6, 90}, {8, 89}, {8, 90}, {9, 89},
    {9, 90}, {10, 89}, {10, 90}, {11, 92}, {11, 93}, {11, 94}, {50, 92}, {50, 93},
    {50, 94}, {51, 92}, {51, 93}, {51, 94}, {53, 92}, {53, 93}, {53, 94}, {54, 92},
    {54, 93}, {54, 94}, {55, 92}, {55, 93}, {55, 94}, {57, 92}, {57, 93}, {57, 94},
    {58, 92}, {58, 93}, {58, 94}, {59, 92}, {59, 93}, {59, 94}, {60, 92}, {60, 93},
    {60, 94}, {62, 92}, {62, 93}, {62, 94}, {63, 92}, {63, 93}, {63, 94}, {65, 92},
    {65, 93}, {65, 94}, {66, 92}, {66, 93}, {66, 94}, {67, 92}, {67, 93}, {67, 94},
    {69, 92}, {69, 93}, {69, 94}, {70, 92}, {70, 93}, {70, 94}, {71, 92}, {71, 93},
    {71, 94}, {72, 92}, {72, 93}, {72, 94}, {47, 92}, {47, 93}, {47, 94}, {48, 92},
    {48, 93}, {48, 94}, {45, 92}, {45, 93}, {45, 94}, {34, 92}, {34, 93}, {34, 94},
    {40, 92}, {40, 93}, {40, 94}, {41, 92}, {41, 93}, {41, 94}, {29, 92}, {29, 93},
    {29, 94}, {31, 92}, {31, 93}, {31, 94}, {32, 92}, {32, 93}, {32, 94}, {33, 92},
    {33, 93}, {33, 94}, {36, 92}, {36, 93}, {36, 94}, {37, 92}, {37, 93}, {37, 94},
    {38, 92}, {38, 93}, {38, 94}, {2, 92}, {2, 93}, {2, 94}, {3, 92}, {3, 93},
    {3, 94}, {43, 92}, {43, 93}, {43, 94}, {44, 92}, {44, 93}, {44, 94}, {1, 92},
    {1, 93}, {1, 94}, {84, 92}, {84, 93}, {84, 94}, {85, 92}, {85, 93}, {85, 94},
    {86, 92}, {86, 93}, {86, 94}, {87, 92}, {87, 93}, {87, 94}, {12, 92}, {12, 93},
    {12, 94}, {14, 92}, {14, 93}, {14, 94}, {15, 92}, {15, 93}, {15, 94}, {16, 92},
    {16, 93}, {16, 94}, {5, 92}, {5, 93}, {5, 94}, {6, 92}, {6, 93}, {6, 94},
    {8, 92}, {8, 93}, {8, 94}, {9, 92}, {9, 93}, {9, 94}, {10, 92}, {10, 93},
    {10, 94}, {11, 96}, {11, 97}, {11, 98}, {11, 99}, {50, 96}, {50, 97}, {50, 98},
    {50, 99}, {51, 96}, {51, 97}, {51, 98}, {51, 99}, {53, 96}, {53, 97}, {53, 98},
    {53, 99}, {54, 96}, {54, 97}, {54, 98}, {54, 99}, {55, 96}, {55, 97}, {55, 98},
    {55, 99}, {57, 96}, {57, 97}, {57, 98}, {57, 99}, {58, 96}, {58, 97}, {58, 98},
    {58, 99}, {59, 96}, {59, 97}, {59, 98}, {59, 99}, {60, 96}, {60, 97}, {60, 98},
    {60, 99}, {62, 96}, {62, 97}, {62, 98}, {62, 99}, {63, 96}, {63, 97}, {63, 98},
    {63, 99}, {65, 96}, {65, 97}, {65, 98}, {65, 99}, {66, 96}, {66, 97}, {66, 98},
    {66, 99}, {67, 96}, {67, 97}, {67, 98}, {67, 99}, {69, 96}, {69, 97}, {69, 98},
    {69, 99}, {70, 96}, {70, 97}, {70, 98}, {70, 99}, {71, 96}, {71, 97}, {71, 98},
    {71, 99}, {72, 96}, {72, 97}, {72, 98}, {72, 99}, {47, 96}, {47, 97}, {47, 98},
    {47, 99}, {48, 96}, {48, 97}, {48, 98}, {48, 99}, {45, 96}, {45, 97}, {45, 98},
    {45, 99}, {34, 96}, {34, 97}, {34, 98}, {34, 99}, {40, 96}, {40, 97}, {40, 98},
    {40, 99}, {41, 96}, {41, 97}, {41, 98}, {41, 99}, {29, 96}, {29, 97}, {29, 98},
    {29, 99}, {31, 96}, {31, 97}, {31, 98}, {31, 99}, {32, 96}, {32, 97}, {32, 98},
    {32, 99}, {33, 96}, {33, 97}, {33, 98}, {33, 99}, {36, 96}, {36, 97}, {36, 98},
    {36, 99}, {37, 96}, {37, 97}, {37, 98}, {37, 99}, {38, 96}, {38, 97}, {38, 98},
    {38, 99}, {2, 96}, {2, 97}, {2, 98}, {2, 99}, {3, 96}, {3, 97}, {3, 98},
    {3, 99}, {43, 96}, {43, 97}, {43, 98}, {43, 99}, {44, 96}, {44, 97}, {44, 98},
    {44, 99}, {1, 96}, {1, 97}, {1, 98}, {1, 99}, {77, 96}, {77, 97}, {77, 98},
    {77, 99}, {78, 96}, {78, 97}, {78, 98}, {78, 99}, {80, 96}, {80, 97}, {80, 98},
    {80, 99}, {81, 96}, {81, 97}, {81, 98}, {81, 99}, {82, 96}, {82, 97}, {82, 98},
    {82, 99}, {84, 96}, {84, 97}, {84, 98}, {84, 99}, {85, 96}, {85, 97}, {85, 98},
    {85, 99}, {86, 96}, {86, 97}, {86, 98}, {86, 99}, {87, 96}, {87, 97}, {87, 98},
    {87, 99}, {17, 96}, {17, 97}, {17, 98}, {17, 99}, {12, 96}, {12, 97}, {12, 98},
    {12, 99}, {14, 96}, {14, 97}, {14, 98}, {14, 99}, {15, 96}, {15, 97}, {15, 98},
    {15, 99}, {16, 96}, {16, 97}, {16, 98}, {16, 99}, {19, 96}, {19, 97}, {19, 98},
    {19, 99}, {20, 96}, {20, 97}, {20, 98}, {20, 99}, {21, 96}, {21, 97}, {21, 98},
    {21, 99}, {5, 96}, {5, 97}, {5, 98}, {5, 99}, {6, 96}, {6, 97}, {6, 98},
    {6, 99}, {8, 96}, {8, 97}, {8, 98}, {8, 99}, {9, 96}, {9, 97}, {9, 98},
    {9, 99}, {10, 96}, {10, 97}, {10, 98}, {10, 99},
};
static const prrtc_sched_def kBaxterSchedule[] = {
    {1, 0}, {0, 0}, {0, 1}, {0, 2}, {0, 3}, {0, 4}, {0, 5}, {0, 6},
    {1, 1}, {1, 2}, {0, 7}, {1, 3}, {1, 4}, {0, 8}, {1, 5}, {1, 6},
    {1, 7}, {1, 8}, {1, 9}, {0, 9}, {1, 10}, {1, 11}, {1, 12}, {1, 13},
    {1, 14}, {1, 15}, {1, 16}, {1, 17}, {0, 10}, {1, 18}, {1, 19}, {1, 20},
    {1, 21}, {1, 22}, {1, 23}, {1, 24}, {1, 25}, {0, 11}, {1, 26}, {1, 27},
    {1, 28}, {1, 29}, {1, 30}, {0, 12}, {0, 13}, {1, 31}, {1, 32}, {1, 33},
    {1, 34}, {1, 35}, {1, 36}, {1, 37}, {1, 38}, {1, 39}, {1, 40}, {1, 41},
    {1, 42}, {1, 43}, {1, 44}, {0, 14}, {1, 45}, {1, 46}, {0, 15}, {1, 47},
    {1, 48}, {1, 49}, {1, 50}, {1, 51}, {1, 52}, {1, 53}, {1, 54}, {1, 55},
    {1, 56}, {1, 57}, {0, 16}, {1, 58}, {1, 59}, {1, 60}, {1, 61}, {1, 62},
    {1, 63}, {1, 64}, {1, 65}, {1, 66}, {1, 67}, {1, 68}, {1, 69}, {1, 70},
    {1, 71}, {1, 72}, {0, 17}, {1, 73}, {1, 74}, {1, 75}, {1, 76}, {1, 77},
    {1, 78}, {1, 79}, {1, 80}, {1, 81}, {1, 82}, {1, 83}, {1, 84}, {1, 85},
    {1, 86}, {1, 87}, {1, 88}, {1, 89}, {1, 90}, {1, 91}, {1, 92}, {1, 93},
    {1, 94}, {1, 95}, {0, 18}, {1, 96}, {0, 19}, {1, 97}, {1, 98}, {1, 99},
    {1, 100}, {1, 101}, {1, 102}, {1, 103}, {1, 104}, {1, 105}, {1, 106}, {1, 107},
    {1, 108}, {1, 109}, {0, 20}, {1, 110}, {1, 111}, {1, 112}, {1, 113}, {1, 114},
    {1, 115}, {1, 116}, {1, 117}, {1, 118}, {1, 119}, {1, 120}, {1, 121}, {1, 122},
    {0, 21}, {1, 123}, {1, 124}, {1, 125}, {1, 126}, {1, 127}, {1, 128}, {1, 129},
    {1, 130}, {1, 131}, {1, 132}, {1, 133}, {1, 134}, {1, 135}, {1, 136}, {0, 22},
    {1, 137}, {1, 138}, {1, 139}, {1, 140}, {1, 141}, {1, 142}, {1, 143}, {1, 144},
    {1, 145}, {1, 146}, {1, 147}, {1, 148}, {1, 149}, {1, 150}, {1, 151}, {1, 152},
    {1, 153}, {0, 23}, {1, 154}, {1, 155}, {1, 156}, {1, 157}, {1, 158}, {1, 159},
    {1, 160}, {1, 161}, {1, 162}, {1, 163}, {1, 164}, {1, 165}, {1, 166}, {1, 167},
    {1, 168}, {0, 24}, {1, 169}, {1, 170}, {1, 171}, {1, 172}, {1, 173}, {1, 174},
    {1, 175}, {1, 176}, {1, 177}, {1, 178}, {1, 179}, {1, 180}, {1, 181}, {1, 182},
    {1, 183}, {1, 184}, {1, 185}, {0, 25}, {1, 186}, {1, 187}, {1, 188}, {1, 189},
    {1, 190}, {1, 191}, {1, 192}, {1, 193}, {1, 194}, {1, 195}, {1, 196}, {1, 197},
    {1, 198}, {1, 199}, {1, 200}, {1, 201}, {1, 202}, {1, 203}, {1, 204}, {1, 205},
    {1, 206}, {1, 207}, {1, 208}, {1, 209}, {1, 210}, {1, 211}, {1, 212}, {1, 213},
    {1, 214}, {1, 215}, {1, 216}, {1, 217}, {0, 26}, {1, 218}, {1, 219}, {1, 220},
    {1, 221}, {1, 222}, {1, 223}, {1, 224}, {1, 225}, {1, 226}, {1, 227}, {1, 228},
    {1, 229}, {1, 230}, {1, 231}, {1, 232}, {1, 233}, {1, 234}, {1, 235}, {1, 236},
    {1, 237}, {0, 27}, {1, 238}, {1, 239}, {1, 240}, {1, 241}, {1, 242}, {1, 243},
    {1, 244}, {1, 245}, {1, 246}, {1, 247}, {1, 248}, {1, 249}, {1, 250}, {1, 251},
    {1, 252}, {1, 253}, {1, 254}, {1, 255}, {1, 256}, {1, 257}, {0, 28}, {1, 258},
    {1, 259}, {1, 260}, {1, 261}, {1, 262}, {1, 263}, {1, 264}, {1, 265}, {1, 266},
    {1, 267}, {1, 268}, {1, 269}, {1, 270}, {1, 271}, {1, 272}, {1, 273}, {1, 274},
    {1, 275}, {1, 276}, {1, 277}, {1, 278}, {0, 29}, {1, 279}, {1, 280}, {1, 281},
    {1, 282}, {1, 283}, {1, 284}, {1, 285}, {1, 286}, {1, 287}, {1, 288}, {1, 289},
    {1, 290}, {1, 291}, {1, 292}, {1, 293}, {1, 294}, {1, 295}, {1, 296}, {1, 297},
    {1, 298}, {1, 299}, {1, 300}, {1, 301}, {1, 302}, {0, 30}, {1, 303}, {1, 304},
    {1, 305}, {1, 306}, {1, 307}, {1, 308}, {1, 309}, {1, 310}, {1, 311}, {1, 312},
    {1, 313}, {1, 314}, {1, 315}, {1, 316}, {1, 317}, {1, 318}, {1, 319}, {1, 320},
    {1, 321}, {1, 322}, {1, 323}, {1, 324}, {0, 31}, {1, 325}, {1, 326}, {1, 327},
    {1, 328}, {1, 329}, {1, 330}, {1, 331}, {1, 332}, {1, 333}, {1, 334}, {1, 335},
    {1, 336}, {1, 337}, {1, 338}, {1, 339}, {1, 340}, {1, 341}, {1, 342}, {1, 343},
    {1, 344}, {1, 345}, {1, 346}, {1, 347}, {1, 348}, {0, 32}, {1, 349}, {1, 350},
    {1, 351}, {1, 352}, {1, 353}, {1, 354},
};
