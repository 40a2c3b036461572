// collision_gb300 - C++ host interface with the reference's names.
//
// A header-only class over the C ABI (collision_gb300.h) that keeps the
// surface of antdvid/Collision's CollisionSolver3d (collid.h:128-244):
// the parameter setters and getters (class statics there, collid.h:180-193;
// per solver here), setDomainBoundary (collid.h:203), resolveCollision
// (collid.h:201) and hasCollision (collid.h:205). assembleFromMesh replaces
// assembleFromInterface (collid.h:242), whose FronTier INTERFACE this library
// does not depend on: it takes the same element lists as flat arrays.
//
// Error behaviour: the reference exits the process on a non-finite value
// (clean_up(ERROR), dcollid.cpp:178-184, 713-718) and raises SIGFPE through
// feenableexcept (dcollid.cpp:320). This class throws collision_gb300::Error
// carrying the cc_status and message instead, and the solver stays usable.
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

#include "collision_gb300.h"

namespace collision_gb300 {

class Error : public std::runtime_error {
public:
    Error(cc_status s, const std::string& msg) : std::runtime_error(msg), status(s) {}
    cc_status status;
};

class CollisionSolver3d {
public:
    explicit CollisionSolver3d(int device = 0) {
        check(cc_create(device, &s_), "cc_create");
        push();
    }
    ~CollisionSolver3d() { cc_destroy(s_); }
    CollisionSolver3d(const CollisionSolver3d&) = delete;
    CollisionSolver3d& operator=(const CollisionSolver3d&) = delete;

    // collid.h:180-193 (defaults dcollid.cpp:28-35)
    void setRoundingTolerance(double v) { p_.eps = v; push(); }
    double getRoundingTolerance() const { return p_.eps; }
    void setFabricThickness(double v) { p_.thickness = v; push(); }
    double getFabricThickness() const { return p_.thickness; }
    void setTimeStepSize(double v) { p_.dt = v; push(); }
    double getTimeStepSize() const { return p_.dt; }
    void setSpringConstant(double v) { p_.k = v; push(); }
    double getSpringConstant() const { return p_.k; }
    void setFrictionConstant(double v) { p_.lambda = v; push(); }
    double getFrictionConstant() const { return p_.lambda; }
    void setPointMass(double v) { p_.m = v; push(); }
    double getPointMass() const { return p_.m; }
    void setRestitutionCoef(double v) { p_.cr = v; push(); }
    double getRestitutionCoef() const { return p_.cr; }

    // collid.h:203
    void setDomainBoundary(const double* L, const double* U) { check(cc_set_domain_boundary(s_, L, U), "domain"); }

    // Replaces assembleFromInterface (collid.h:242): triangles of every
    // non-boundary surface, then the bonds of every string curve, in the
    // reference's hseList order (dcollid3d.cpp:25-43).
    void assembleFromMesh(int n_points, const std::vector<int32_t>& tris, const std::vector<int32_t>& tri_surface,
                          const std::vector<double>& tri_rest_len, const std::vector<int32_t>& bonds,
                          const std::vector<double>& bond_rest_len, const std::vector<uint8_t>& fixed) {
        cc_mesh m;
        m.n_points = n_points;
        m.n_tris = (int32_t)(tris.size() / 3);
        m.tris = tris.data();
        m.tri_surface = tri_surface.empty() ? nullptr : tri_surface.data();
        m.tri_rest_len = tri_rest_len.data();
        m.n_bonds = (int32_t)(bonds.size() / 2);
        m.bonds = bonds.data();
        m.bond_rest_len = bond_rest_len.data();
        m.fixed = fixed.empty() ? nullptr : fixed.data();
        check(cc_assemble(s_, &m), "assemble");
        n_points_ = n_points;
    }

    // collid.h:201. x_old / x_cand: positions at the start of the step and
    // candidate positions; vel and has_collsn in/out; x_out the result.
    void resolveCollision(const double* x_old, const double* x_cand, double* vel, uint8_t* has_collsn,
                          double* x_out) {
        int hc = 0;
        check(cc_resolve(s_, x_old, x_cand, vel, has_collsn, x_out, &hc), "resolveCollision");
        has_collision_ = hc != 0;
    }

    // collid.h:205
    bool hasCollision() const { return has_collision_; }

    cc_solver* handle() { return s_; }

private:
    void push() { check(cc_set_params(s_, &p_), "params"); }
    void check(cc_status st, const char* what) {
        if (st == CC_OK) return;
        char buf[512] = {0};
        if (s_) cc_last_error(s_, buf, sizeof(buf));
        throw Error(st, std::string(what) + ": " + buf);
    }
    cc_solver* s_ = nullptr;
    cc_params p_{1e-3, 1e-4, 1e-6, 1000.0, 0.01, 0.02, 0.0};
    bool has_collision_ = false;
    int n_points_ = 0;
};

}  // namespace collision_gb300
