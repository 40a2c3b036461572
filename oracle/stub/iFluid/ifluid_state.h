/*
 * Per-point state record expected by the collision sources (collid.h:20-39
 * documents the required fields; dcollid.cpp and dcollid3d.cpp also use
 * collsnImpulse_RG, collsn_num_RG and is_movableRG). Test infrastructure only.
 */
#ifndef ORACLE_STUB_IFLUID_STATE_H
#define ORACLE_STUB_IFLUID_STATE_H
struct UF {
    POINT* next_pt;
    POINT* root;
    POINT* tail;
    int num_pts;
};

struct STATE {
    double vel[3];
    double collsnImpulse[3];
    double collsnImpulse_RG[3];
    double friction[3];
    double avgVel[3];
    double x_old[3];
    int collsn_num;
    int collsn_num_RG;
    bool has_collsn;
    bool is_fixed;
    bool is_movableRG;
    UF impZone;
};
#endif
