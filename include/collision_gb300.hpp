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

    // A movable rigid body's HYPER_SURF data (total_mass, center_of_mass,
    // center_of_mass_velo) in, and after a step the centre of mass and its
    // velocity updateFinalForRG (dcollid.cpp:626-675) wrote.
    void setBody(int surface, double mass, const double* com, const double* comv) {
        check(cc_set_body(s_, 0, surface, mass, com, comv), "body");
    }
    void body(int surface, double* com, double* comv) { check(cc_get_body(s_, 0, surface, com, comv), "body"); }

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

    // Arithmetic of the narrow phase (0 plain FP64, 1 mixed precision with
    // the same results), launch tuning and the last step's counters; none of
    // these changes results (cc_set_mode, cc_autotune, cc_set_tuning,
    // cc_get_counters).
    void setMode(int mode) { check(cc_set_mode(s_, mode), "mode"); }
    double autotune() {
        double ms = 0.0;
        check(cc_autotune(s_, &ms), "autotune");
        return ms;
    }
    void setTuning(int knob, int value) { check(cc_set_tuning(s_, knob, value), "tuning"); }
    int tuning(int knob) { return cc_get_tuning(s_, knob); }
    std::vector<long long> counters() {
        std::vector<long long> c(64);
        c.resize((size_t)cc_get_counters(s_, c.data(), (int)c.size()));
        return c;
    }

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

// Many independent scenes in one solver (cc_assemble_batch): each scene is
// what one CollisionSolver3d holds, with its own parameters and domain box.
// Point arrays of the resolve call hold scene 0's points, then scene 1's...
class SceneBatch {
public:
    struct Mesh {
        int n_points = 0;
        std::vector<int32_t> tris, tri_surface;
        std::vector<double> tri_rest_len;
        std::vector<int32_t> bonds;
        std::vector<double> bond_rest_len;
        std::vector<uint8_t> fixed;
    };

    explicit SceneBatch(int device = 0) { check(cc_create(device, &s_), "cc_create"); }
    ~SceneBatch() { cc_destroy(s_); }
    SceneBatch(const SceneBatch&) = delete;
    SceneBatch& operator=(const SceneBatch&) = delete;

    void assemble(const std::vector<Mesh>& meshes) {
        std::vector<cc_mesh> ms(meshes.size());
        for (size_t i = 0; i < meshes.size(); ++i) {
            const Mesh& m = meshes[i];
            ms[i].n_points = m.n_points;
            ms[i].n_tris = (int32_t)(m.tris.size() / 3);
            ms[i].tris = m.tris.data();
            ms[i].tri_surface = m.tri_surface.empty() ? nullptr : m.tri_surface.data();
            ms[i].tri_rest_len = m.tri_rest_len.data();
            ms[i].n_bonds = (int32_t)(m.bonds.size() / 2);
            ms[i].bonds = m.bonds.data();
            ms[i].bond_rest_len = m.bond_rest_len.data();
            ms[i].fixed = m.fixed.empty() ? nullptr : m.fixed.data();
        }
        check(cc_assemble_batch(s_, ms.data(), (int)ms.size()), "assemble_batch");
        n_ = (int)meshes.size();
        point_off_.assign((size_t)n_ + 1, 0);
        check(cc_get_scene_offsets(s_, point_off_.data(), nullptr), "scene offsets");
        has_collision_.assign((size_t)n_, 0);
        status_.assign((size_t)n_, 0);
    }
    int numScenes() const { return n_; }
    // first point of each scene; the last entry is the total
    const std::vector<int32_t>& pointOffsets() const { return point_off_; }

    void setParams(int scene, const cc_params& p) { check(cc_set_scene_params(s_, scene, &p), "scene params"); }
    void setParams(const cc_params& p) { check(cc_set_params(s_, &p), "params"); }
    void setDomainBoundary(int scene, const double* L, const double* U) {
        check(cc_set_scene_domain_boundary(s_, scene, L, U), "scene domain");
    }
    void setZoneCap(int cap) { check(cc_set_zone_cap(s_, cap), "zone cap"); }
    void setBody(int scene, int surface, double mass, const double* com, const double* comv) {
        check(cc_set_body(s_, scene, surface, mass, com, comv), "body");
    }
    void body(int scene, int surface, double* com, double* comv) {
        check(cc_get_body(s_, scene, surface, com, comv), "body");
    }
    void setSceneEnabled(int scene, bool on) { check(cc_set_scene_enabled(s_, scene, on ? 1 : 0), "enable"); }

    // resolveCollision on every scene (host arrays over all points). Returns
    // false when some scene stopped at the impact-zone cap (see status()).
    bool resolveCollision(const double* x_old, const double* x_cand, double* vel, uint8_t* has_collsn,
                          double* x_out) {
        cc_status st = cc_resolve_batch(s_, x_old, x_cand, vel, has_collsn, x_out, has_collision_.data());
        if (st != CC_ITER_CAP) check(st, "resolve_batch");
        check(cc_get_scene_status(s_, status_.data()), "scene status");
        return st == CC_OK;
    }
    bool hasCollision(int scene) const { return has_collision_[(size_t)scene] != 0; }
    int status(int scene) const { return status_[(size_t)scene]; }

    // Arithmetic of the narrow phase (0 plain FP64, 1 mixed precision with
    // the same results), launch tuning and the last step's counters; none of
    // these changes results (cc_set_mode, cc_autotune, cc_set_tuning,
    // cc_get_counters).
    void setMode(int mode) { check(cc_set_mode(s_, mode), "mode"); }
    double autotune() {
        double ms = 0.0;
        check(cc_autotune(s_, &ms), "autotune");
        return ms;
    }
    void setTuning(int knob, int value) { check(cc_set_tuning(s_, knob, value), "tuning"); }
    int tuning(int knob) { return cc_get_tuning(s_, knob); }
    std::vector<long long> counters() {
        std::vector<long long> c(64);
        c.resize((size_t)cc_get_counters(s_, c.data(), (int)c.size()));
        return c;
    }

    cc_solver* handle() { return s_; }

private:
    void check(cc_status st, const char* what) {
        if (st == CC_OK) return;
        char buf[512] = {0};
        if (s_) cc_last_error(s_, buf, sizeof(buf));
        throw Error(st, std::string(what) + ": " + buf);
    }
    cc_solver* s_ = nullptr;
    int n_ = 0;
    std::vector<int32_t> point_off_;
    std::vector<int> has_collision_, status_;
};

}  // namespace collision_gb300
