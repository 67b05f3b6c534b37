// TEST INFRASTRUCTURE ONLY (the oracle).
//
// CPU FP64 restatement of sdfibm's fluid-solid coupling path, used by tests/, __graft_entry__.smoke() and the
// cpu_baseline leg of bench.py to check the GPU path and as the timed CPU baseline; nothing in the product loads it.
// It follows the reference line by line:
//   SolidCloud::interact / solidFluidInteract / checkAlpha / fixInternal / evolve / addMidEnvironment /
//   solidSolidInteract / solidSolidCollision   src/solidcloud.cpp:288-301, 361-433, 435-464, 466-570
//   SolidCloud::calcMeanField                   src/solidcloud.cpp:315-359
//   CellEnumerator                              src/cellenumerator.cpp:6-78, src/cellenumerator.h:41-52
//   GeometricTools                              src/geometrictools.cpp:6-116
//   Solid                                       src/solid.h:109-202
//   UGrid, collision laws                       src/libcollision/ugrid.cpp:5-77, ugrid.h:46-57, collision.cpp:7-57
//   motions                                     src/libmotion/*.h (constraint bodies)
//   forcers                                     src/libforcer/{constant,spring,magnetic}.h (generate bodies)
// Two modes with identical arithmetic:
//   faithful: the reference's data structures (per-solid O(N) type array, std::queue, std::set per type,
//             std::function predicate, unordered_map phi cache, full-mesh seed fallback scan, full-mesh
//             nearest-cell search and dense field reset) -- the timed CPU baseline;
//   fast:     bbox-local hash sets and local nearest-cell search, for large meshes.
// Parity anchors: the golden As of examples/flow_past_cylinder/re200/0/As and the OpenFOAM ordering conventions of
// examples/falling_ellipse/constant/polyMesh (fixtures under tests/golden/).  Collision, evolve, motions and
// forcers have no reference test or golden vector: that part is parity unpinned beyond this restatement.
// Compile with -ffp-contract=off (no FMA contraction) so x86 and Arm builds give the same bits.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <limits>
#include <memory>
#include <queue>
#include <set>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../include/sdfibm_cuda.h"
#include "oracle_math.h"
#include "oracle_mesh.h"
#include "oracle_shapes.h"

namespace oracle {

enum CELL_TYPE { UNVISITED = 0, ALL_INSIDE = 1, CENTER_INSIDE = 2, CENTER_OUTSIDE = 3, ALL_OUTSIDE = 4 };

struct Solid {
    sdfibm_solid_desc d;
    int id;
    V3 center;
    Quat q;
    V3 vel, omega, force, torque;
    V3 fluid_force, fluid_torque, fluid_force_old, fluid_torque_old;
    V3 forcer_force, forcer_torque, forcer_force_old, forcer_torque_old;
    bool first_fluid_step = true, first_forcer_step = true;
    T33 moi_inv;

    // Solid::phi01 / Solid::phi (solid.h:109-119)
    bool phi01(const V3& p) const { return shapeInside(d.shape, world2local(p, center, q)); }
    double phi(const V3& p) const { return shapeSDF(d.shape, world2local(p, center, q)); }
    // Solid::evalPointVelocity (solid.h:121-124)
    V3 evalPointVelocity(const V3& p) const { return vel + cross(omega, p - center); }
};

inline V3 arr3(const double* a) { return V3{a[0], a[1], a[2]}; }

// double -> integer by truncation with the device's conversion rules (NaN -> 0, out of range -> the nearest limit):
// a non-finite or far-off solid position then has one defined result on every host (a plain cast is undefined there)
template <class I> inline I to_int_rz(double t) {
    if (!(t == t)) return 0;
    if (t >= (double)std::numeric_limits<I>::max()) return std::numeric_limits<I>::max();
    if (t <= (double)std::numeric_limits<I>::min()) return std::numeric_limits<I>::min();
    return (I)t;
}
inline void put3(double* a, const V3& v) { a[0] = v.x; a[1] = v.y; a[2] = v.z; }

// ---- motions: IMotion::constraint ----------------------------------------------------------------------------
static void motionConstraint(const Solid& s, double time, V3& velocity, V3& omega) {
    const double* p = s.d.motion_p;
    switch (s.d.motion_type) {
        case SDFIBM_MOTION_FREE: return;
        case SDFIBM_MOTION_000002:  // motion000002.h:22-27
            velocity = V3{0, 0, 0}; omega = V3{0, 0, 0}; omega.z = p[1]; return;
        case SDFIBM_MOTION_110002:  // motion110002.h:22-27
            velocity.z = 0.0; omega = V3{0, 0, 0}; omega.z = p[1]; return;
        case SDFIBM_MOTION_222000:  // motion222000.h:22-26
            velocity = V3{p[0], p[1], p[2]}; omega = V3{0, 0, 0}; return;
        case SDFIBM_MOTION_SINEDIRECTIONAL:  // motionsinedirectional.h:28-32
            velocity = p[0] * p[2] * std::cos(p[2] * time) * V3{p[3], p[4], p[5]}; omega = V3{0, 0, 0}; return;
        case SDFIBM_MOTION_01MASK:  // motion01mask.h:50-54
            velocity = cmptMultiply(velocity, V3{p[0], p[1], p[2]});
            omega = cmptMultiply(omega, V3{p[3], p[4], p[5]});
            return;
        case SDFIBM_MOTION_ROTOR:  // motionrotor.h:40-47
            velocity = V3{0, 0, 0};
            velocity.x = -p[2] * p[1] * std::sin(p[1] * time + p[3]);
            velocity.y = p[2] * p[1] * std::cos(p[1] * time + p[3]);
            omega = V3{0, 0, 0}; omega.z = p[4];
            return;
        case SDFIBM_MOTION_OPENCLOSE: {  // motionopenclose.h:16-40
            double t = std::fmod(time, 5.0), v = 0.0;
            if (t > 1 && t < 2) v = -1.0;
            if (t > 3 && t < 4) v = 1.0;
            velocity = V3{0, v, 0}; omega = V3{0, 0, 0};
            return;
        }
    }
}

// ---- forcers: IForcer::generate --------------------------------------------------------------------------------
static void forcerGenerate(const Solid& s, double time, V3& f, V3& t) {
    const double* p = s.d.forcer_p;
    switch (s.d.forcer_type) {
        case SDFIBM_FORCER_CONSTANT: f = V3{p[0], p[1], p[2]}; t = V3{p[3], p[4], p[5]}; return;
        case SDFIBM_FORCER_SPRING: {  // spring.h:35-46
            V3 r = s.center - V3{p[0], p[1], p[2]};
            V3 force{0, 0, 0};
            if (mag(r) > SMALL) force = -p[3] * r * (1.0 - p[4] / mag(r));
            f = force; t = V3{0, 0, 0};
            return;
        }
        case SDFIBM_FORCER_MAGNETIC: {  // magnetic.h:28-41
            const V3 m_original = (1.0) * (V3{0.0, 0.0, 1.0});
            V3 B = p[3] * std::cos(p[4] * time) * V3{p[0], p[1], p[2]};
            V3 m = transform(conjugate(s.q), m_original);
            f = V3{0, 0, 0}; t = cross(m, B);
            return;
        }
        default: f = V3{0, 0, 0}; t = V3{0, 0, 0}; return;
    }
}

// ---- the cloud --------------------------------------------------------------------------------------------------
struct CloudBase {
    virtual ~CloudBase() = default;
    virtual int interact(double time, double dt, const double* U, double* As, double* Fs, double* Ts, int32_t* Ct,
                         double* FT) = 0;
    virtual int interactThreads(double dt, const double* U, double* As, double* Fs, double* Ts, int32_t* Ct,
                                double* FT, int nthreads) = 0;
    virtual int64_t touched(int s, int64_t* cells, int8_t* types, int64_t cap) const = 0;
    virtual int fixInternal(const int32_t* Ct, double* U) const = 0;
    virtual int64_t nCells() const = 0;
    virtual void cellCentre(int64_t c, double* out) const = 0;
    virtual double cellFraction(int s, int64_t c, int method) = 0;
    virtual int meanField(const sdfibm_shape_desc& sampler, const double* U, int32_t* Ct, double* out) = 0;

    std::vector<Solid> solids;
    sdfibm_options opt{};
    int twod = 0;
    bool faithful = true;
    double last_seconds = 0.0;
    int64_t last_pairs = 0;
    std::vector<std::vector<int64_t>> touched_cells;
    std::vector<std::vector<int8_t>> touched_types;
    V3 bmin, bmax;

    void setState(int i, const sdfibm_solid_state& st) {
        Solid& s = solids[i];
        s.center = arr3(st.pos); s.q = Quat{st.quat[0], arr3(st.quat + 1)};
        s.vel = arr3(st.vel); s.omega = arr3(st.omega); s.force = arr3(st.force); s.torque = arr3(st.torque);
        s.fluid_force = arr3(st.fluid_force); s.fluid_torque = arr3(st.fluid_torque);
        s.fluid_force_old = arr3(st.fluid_force_old); s.fluid_torque_old = arr3(st.fluid_torque_old);
        s.forcer_force = arr3(st.forcer_force); s.forcer_torque = arr3(st.forcer_torque);
        s.forcer_force_old = arr3(st.forcer_force_old); s.forcer_torque_old = arr3(st.forcer_torque_old);
        s.first_fluid_step = st.first_fluid_step != 0; s.first_forcer_step = st.first_forcer_step != 0;
    }
    void getState(int i, sdfibm_solid_state& st) const {
        const Solid& s = solids[i];
        put3(st.pos, s.center); st.quat[0] = s.q.w; put3(st.quat + 1, s.q.v);
        put3(st.vel, s.vel); put3(st.omega, s.omega); put3(st.force, s.force); put3(st.torque, s.torque);
        put3(st.fluid_force, s.fluid_force); put3(st.fluid_torque, s.fluid_torque);
        put3(st.fluid_force_old, s.fluid_force_old); put3(st.fluid_torque_old, s.fluid_torque_old);
        put3(st.forcer_force, s.forcer_force); put3(st.forcer_torque, s.forcer_torque);
        put3(st.forcer_force_old, s.forcer_force_old); put3(st.forcer_torque_old, s.forcer_torque_old);
        st.first_fluid_step = s.first_fluid_step; st.first_forcer_step = s.first_forcer_step;
    }

    // Solid::move (solid.h:181-202)
    void move(Solid& s, double time, double dt) {
        V3 velocity_old = s.vel;
        V3 omega_old = s.omega;
        s.vel += s.force * s.d.mass_inv * dt;
        T33 R = rotation(s.q);
        T33 moi_inv_world = dotTT(dotTT(R, s.moi_inv), transpose(R));
        s.omega += dotTV(moi_inv_world, s.torque) * dt;
        if (s.d.motion_type != SDFIBM_MOTION_FREE) motionConstraint(s, time, s.vel, s.omega);
        s.center += 0.5 * (s.vel + velocity_old) * dt;
        Quat dq = 0.5 * Quat{0.0, 0.5 * (s.omega + omega_old)} * s.q * dt;
        s.q = Quat{s.q.w + dq.w, s.q.v + dq.v};
        s.q = normalise(s.q);
    }

    // collision (solidcloud.cpp:492-519, collision.cpp:7-35)
    static double planeSphere(const Solid& p, const Solid& s, V3& cP, V3& cN) {
        V3 s_center = transform(conjugate(p.q), s.center - p.center);
        double p2s = s_center.y;
        cN = transform(p.q, V3{0, 1, 0});
        cP = s.center - s.d.shape.radiusB * cN;
        return s.d.shape.radiusB - p2s;
    }
    static double sphereSphere(const Solid& s1, const Solid& s2, V3& cP, V3& cN) {
        V3 s2s = s2.center - s1.center;
        cN = normalised(s2s);
        double r1 = s1.d.shape.radiusB, r2 = s2.d.shape.radiusB;
        cP = 0.5 * (s1.center + s2.center + (r1 - r2) * cN);
        return r1 + r2 - mag(s2s);
    }
    int collisionId(const Solid& s) const {
        if (opt.collision_mode == SDFIBM_COLLISION_SPHERES) return s.d.shape.type == SDFIBM_SHAPE_PLANE ? 0 : 2;
        return s.d.shape.collision_id;
    }
    void solidSolidCollision(Solid& s1, Solid& s2) {
        int a = collisionId(s1), b = collisionId(s2);
        double cd;
        V3 cP, cN;
        if ((a == 1 || a == 2) && b == 0) cd = planeSphere(s2, s1, cP, cN);        // circlePlane, spherePlane
        else if (a == 0 && (b == 1 || b == 2)) cd = planeSphere(s1, s2, cP, cN);   // planeCircle, planeSphere
        else if ((a == 1 && b == 1) || (a == 2 && b == 2)) cd = sphereSphere(s1, s2, cP, cN);
        else return;  // no entry in collisionFuncTable
        if (cd < 0) return;
        V3 force = 1e4 * cd * cN;
        V3 torque{0, 0, 0};
        s1.force += -force; s1.torque += -torque;
        s2.force += force; s2.torque += torque;
    }
    // solidSolidInteract with UGrid(bbox, 2*radiusB) (solidcloud.cpp:477-490, ugrid.cpp:5-77)
    void solidSolidInteract() {
        last_pairs = 0;
        if (opt.collision_mode == SDFIBM_COLLISION_OFF) return;
        double rB = -1.0;
        for (const Solid& s : solids) rB = std::max(rB, s.d.shape.radiusB);
        double delta = 2 * rB;
        if (!(delta > 0)) return;
        double dINV = 1.0 / delta;
        double low[3] = {bmin.x, bmin.y, bmin.z}, high[3] = {bmax.x, bmax.y, bmax.z};
        int nx = to_int_rz<int>(std::ceil((high[0] - low[0]) * dINV));
        int ny = to_int_rz<int>(std::ceil((high[1] - low[1]) * dINV));
        int nz = to_int_rz<int>(std::ceil((high[2] - low[2]) * dINV));
        if (nx <= 0 || ny <= 0 || nz <= 0) return;
        int64_t nynz = (int64_t)ny * nz;
        int64_t ncell = (int64_t)nx * ny * nz;
        std::unordered_map<int64_t, std::vector<int>> map;
        for (const Solid& s : solids) {
            int i = to_int_rz<int>(std::floor((s.center.x - low[0]) * dINV));
            int j = to_int_rz<int>(std::floor((s.center.y - low[1]) * dINV));
            int k = to_int_rz<int>(std::floor((s.center.z - low[2]) * dINV));
            map[(int64_t)i * nynz + (int64_t)j * nz + k].push_back(s.id);
        }
        std::vector<std::pair<int, int>> pairs;
        for (int i = 0; i < nx; ++i)
            for (int j = 0; j < ny; ++j)
                for (int k = 0; k < nz; ++k) {
                    int64_t myid = (int64_t)i * nynz + (int64_t)j * nz + k;
                    auto it = map.find(myid);
                    if (it == map.end() || it->second.empty()) continue;
                    for (int nbi = i - 1; nbi <= i + 1; ++nbi)
                        for (int nbj = j - 1; nbj <= j + 1; ++nbj)
                            for (int nbk = k - 1; nbk <= k + 1; ++nbk) {
                                if (nbi < 0 || nbi > nx - 1) continue;
                                if (nbj < 0 || nbj > ny - 1) continue;
                                if (nbk < 0 || nbk > nz - 1) continue;
                                int64_t nbid = (int64_t)nbi * nynz + (int64_t)nbj * nz + nbk;
                                auto jt = map.find(nbid);
                                if (jt == map.end() || jt->second.empty()) continue;
                                for (int pi : it->second)
                                    for (int qi : jt->second)
                                        if (pi < qi) pairs.emplace_back(pi, qi);
                            }
                }
        (void)ncell;
        last_pairs = (int64_t)pairs.size();
        for (auto& pr : pairs) solidSolidCollision(solids[pr.first], solids[pr.second]);
    }

    // SolidCloud::evolve (solidcloud.cpp:521-562)
    int evolve(double time, double dt) {
        int N = opt.n_subiter > 0 ? opt.n_subiter : (solids.size() == 1 ? 1 : 20);
        double dt_sub = dt / N;
        const V3 g = arr3(opt.gravity);
        for (int it = 0; it < N; ++it) {
            for (Solid& s : solids) { s.force = V3{0, 0, 0}; s.torque = V3{0, 0, 0}; }
            for (Solid& s : solids) {  // Solid::applyForcer (solid.h:148-163)
                if (s.d.forcer_type == SDFIBM_FORCER_NONE) continue;
                V3 f_, t_;
                forcerGenerate(s, time, f_, t_);
                s.forcer_force = f_; s.forcer_torque = t_;
                if (s.first_forcer_step) {
                    s.forcer_force_old = s.forcer_force; s.forcer_torque_old = s.forcer_torque;
                    s.first_forcer_step = false;
                }
                s.force += (1.5 * s.forcer_force - 0.5 * s.forcer_force_old);
                s.torque += (1.5 * s.forcer_torque - 0.5 * s.forcer_torque_old);
            }
            for (Solid& s : solids) {  // Solid::addMidFluidForceAndTorque (solid.h:164-174)
                if (s.first_fluid_step) {
                    s.fluid_force_old = s.fluid_force; s.fluid_torque_old = s.fluid_torque;
                    s.first_fluid_step = false;
                }
                s.force += (1.5 * s.fluid_force - 0.5 * s.fluid_force_old);
                s.torque += (1.5 * s.fluid_torque - 0.5 * s.fluid_torque_old);
            }
            for (Solid& s : solids) {  // addMidEnvironment (solidcloud.cpp:466-475), Solid::addAcceleration
                double rhos = s.d.rho;
                V3 gprime = ((rhos - opt.rho_f) / rhos) * g;
                s.force += s.d.mass * gprime;
            }
            solidSolidInteract();
            for (Solid& s : solids) move(s, time, dt_sub);
        }
        for (Solid& s : solids) {  // storeOldForce (solid.h:141-147)
            s.fluid_force_old = s.fluid_force; s.fluid_torque_old = s.fluid_torque;
            s.forcer_force_old = s.forcer_force; s.forcer_torque_old = s.forcer_torque;
        }
        return 0;
    }
};

template <class M>
struct Cloud : CloudBase {
    const M& mesh;
    std::unique_ptr<M> owned;

    Cloud(std::unique_ptr<M> m, const sdfibm_solid_desc* sd, int n, const sdfibm_options& o, bool faith)
        : mesh(*m), owned(std::move(m)) {
        opt = o;
        faithful = faith;
        for (int i = 0; i < n; ++i) {
            Solid s;
            s.d = sd[i];
            s.id = i;
            s.center = arr3(sd[i].pos);
            s.q = Quat{sd[i].quat[0], arr3(sd[i].quat + 1)};
            s.vel = arr3(sd[i].vel); s.omega = arr3(sd[i].omega);
            s.force = s.torque = s.fluid_force = s.fluid_torque = V3{0, 0, 0};
            s.fluid_force_old = s.fluid_torque_old = s.forcer_force = s.forcer_torque = V3{0, 0, 0};
            s.forcer_force_old = s.forcer_torque_old = V3{0, 0, 0};
            const double* m = sd[i].moi_inv;
            s.moi_inv = T33{m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8]};
            solids.push_back(s);
        }
        touched_cells.resize(n);
        touched_types.resize(n);
    }
    int64_t nCells() const override { return mesh.nCells(); }

    // meshSearch::findNearestCell: nearest cell centre, ties to the lowest label (linear-search semantics)
    int64_t findNearestCell(const V3& p) const;

    // CellEnumerator::CountVertexInside (cellenumerator.cpp:36-45)
    template <class Pred>
    int countVertexInside(int64_t c, const Pred& pred) const;

    // GeometricTools (geometrictools.cpp)
    struct Geo {
        const Cloud& cl;
        std::unordered_map<int64_t, double> cache;
        explicit Geo(const Cloud& c) : cl(c) {}
        double updateCache(int64_t v, const Solid& s) {
            auto it = cache.find(v);
            if (it == cache.end()) { double ph = s.phi(cl.point(v)); cache[v] = ph; return ph; }
            return it->second;
        }
        static double lineFraction(double pa, double pb) {
            if (pa > 0 && pb > 0) return 0;
            if (pa <= 0 && pb <= 0) return 1;
            if (pa > 0) return -pb / (pa - pb);
            return -pa / (pb - pa);
        }
        V3 apex(const int64_t* v, int n) {
            const V3 A = cl.point(v[0]);
            double phiA = cache[v[0]];
            V3 B{0, 0, 0};
            double phiB = 0.0;
            for (int i = 1; i < n; ++i) {
                B = cl.point(v[i]);
                phiB = cache[v[i]];
                if (phiA * phiB <= 0) break;
            }
            return A - std::abs(phiA) / (SMALL + std::fabs(phiA) + std::fabs(phiB)) * (A - B);
        }
        double faceArea(const int64_t* v, int n) {
            V3 ap = apex(v, n);
            std::vector<double> phiarr(n);  // heap vector per face, as geometrictools.cpp:80
            for (int i = 0; i < n; ++i) phiarr[i] = cache[v[i]];
            double area = 0.0;
            for (int iseg = 0; iseg < n; ++iseg) {
                const double phiO = phiarr[iseg];
                const double phiA = phiarr[(iseg + 1) % n];
                const V3 O = cl.point(v[iseg]);
                const V3 A = cl.point(v[(iseg + 1) % n]);
                area += std::fabs(0.5 * mag(cross(A - O, ap - O))) * lineFraction(phiO, phiA);
            }
            return area;
        }
        double faceAreaFraction(const int64_t* v, int n, const V3& Sf) {
            int sign_sum = 0;
            for (int i = 0; i < n; ++i) {
                if (cache[v[i]] > 0) ++sign_sum; else --sign_sum;
            }
            if (sign_sum == n) return 0.0;
            if (sign_sum == -n) return 1.0;
            return faceArea(v, n) / mag(Sf);
        }
        double cellVolume(int64_t c, const Solid& s, bool isTWOD) {
            int64_t vi[8];
            int nv = cl.cellPointsOf(c, vi);
            for (int i = 0; i < nv; ++i) updateCache(vi[i], s);
            V3 ap = apex(vi, nv);
            if (isTWOD) ap.z = 0.0;
            double volume = 0.0;
            FaceRef fr[12];
            int nf = cl.cellFacesOf(c, fr);
            for (int f = 0; f < nf; ++f) {
                double eps_f = faceAreaFraction(fr[f].v, 4, fr[f].Sf);
                volume += (1.0 / 3.0) * eps_f * std::fabs(dot(ap - fr[f].Cf, fr[f].Sf));
            }
            return volume;
        }
    };

    V3 point(int64_t p) const;
    int cellPointsOf(int64_t c, int64_t* out) const;
    int cellFacesOf(int64_t c, FaceRef* out) const;
    int cellCellsOf(int64_t c, int64_t* out) const;
    V3 centre(int64_t c) const;
    double vol(int64_t c) const;
    void cellCentre(int64_t c, double* out) const override { put3(out, centre(c)); }

    // conservative cell-index box of the cells that can hold an inside vertex (fast mode); false = whole mesh
    bool bboxCells(const Solid& s, int64_t lo[3], int64_t hi[3]) const;

    // CellEnumerator: returns the three sorted sets; order (optional) receives the touched cells with their types in
    // the enumerator's queue order (CellEnumerator::Next / GetCurCellInd, cellenumerator.h:41-60)
    void enumerate(const Solid& s, std::vector<int64_t>& inside, std::vector<int64_t>& cin,
                   std::vector<int64_t>& cout, std::vector<std::pair<int64_t, int8_t>>* order = nullptr) const {
        auto pred = [&](const V3& v) { return s.phi01(v); };
        int64_t seed = findNearestCell(s.center);
        inside.clear(); cin.clear(); cout.clear();
        if (order) order->clear();
        if (faithful) {
            std::function<bool(const V3&)> fpred = pred;
            std::vector<int> m_ct(mesh.nCells(), UNVISITED);  // cellenumerator.cpp:49
            std::unordered_map<int, std::set<size_t>> is_;
            std::queue<int64_t> q;
            if (countVertexInside(seed, fpred) == 0) {
                seed = -1;
                for (int64_t c = 0; c < mesh.nCells(); ++c)
                    if (countVertexInside(c, fpred) > 0) { seed = c; break; }
            }
            if (seed >= 0) {
                q.push(seed);
                int64_t tmp[8];
                int nv = cellPointsOf(seed, tmp);
                if (countVertexInside(seed, fpred) == nv) m_ct[seed] = ALL_INSIDE;
                else if (fpred(centre(seed))) m_ct[seed] = CENTER_INSIDE;
                else m_ct[seed] = CENTER_OUTSIDE;
                is_[m_ct[seed]].insert(seed);
            }
            while (!q.empty()) {
                int64_t icur = q.front();
                if (order) order->emplace_back(icur, (int8_t)m_ct[icur]);
                int64_t nb[6];
                int nn = cellCellsOf(icur, nb);
                int64_t tmp[8];
                int nvc = cellPointsOf(icur, tmp);
                for (int t = 0; t < nn; ++t) {
                    int64_t inb = nb[t];
                    if (m_ct[inb] != UNVISITED) continue;
                    int n_in = countVertexInside(inb, fpred);
                    if (n_in == 0) { m_ct[inb] = ALL_OUTSIDE; is_[m_ct[inb]].insert(inb); continue; }
                    q.push(inb);
                    if (n_in == nvc) m_ct[inb] = ALL_INSIDE;
                    else if (fpred(centre(inb))) m_ct[inb] = CENTER_INSIDE;
                    else m_ct[inb] = CENTER_OUTSIDE;
                    is_[m_ct[inb]].insert(inb);
                }
                q.pop();
            }
            for (auto c : is_[ALL_INSIDE]) inside.push_back((int64_t)c);
            for (auto c : is_[CENTER_INSIDE]) cin.push_back((int64_t)c);
            for (auto c : is_[CENTER_OUTSIDE]) cout.push_back((int64_t)c);
            return;
        }
        // fast mode: same BFS semantics, visited set in a hash map, seed fallback scan limited to the bbox
        std::unordered_map<int64_t, int8_t> ct;
        auto typeOf = [&](int64_t c, int n_in, int nv) -> int8_t {
            if (n_in == nv) return ALL_INSIDE;
            return pred(centre(c)) ? CENTER_INSIDE : CENTER_OUTSIDE;
        };
        auto centreType = [&](int64_t c) -> int8_t { return pred(centre(c)) ? CENTER_INSIDE : CENTER_OUTSIDE; };
        if (countVertexInside(seed, pred) == 0) {
            seed = -1;
            int64_t lo[3], hi[3];
            if (bboxCells(s, lo, hi)) {
                for (int64_t k = lo[2]; k <= hi[2] && seed < 0; ++k)
                    for (int64_t j = lo[1]; j <= hi[1] && seed < 0; ++j)
                        for (int64_t i = lo[0]; i <= hi[0]; ++i) {
                            int64_t c = cellIndex(i, j, k);
                            if (countVertexInside(c, pred) > 0) { seed = c; break; }
                        }
            } else {
                for (int64_t c = 0; c < mesh.nCells(); ++c)
                    if (countVertexInside(c, pred) > 0) { seed = c; break; }
            }
        }
        if (seed < 0) return;
        std::vector<int64_t> q;
        {
            int64_t tmp[8];
            int nv = cellPointsOf(seed, tmp);
            ct[seed] = typeOf(seed, countVertexInside(seed, pred), nv);
            q.push_back(seed);
        }
        for (size_t h = 0; h < q.size(); ++h) {
            int64_t icur = q[h];
            int64_t nb[6];
            int nn = cellCellsOf(icur, nb);
            int64_t tmp[8];
            int nvc = cellPointsOf(icur, tmp);
            for (int t = 0; t < nn; ++t) {
                int64_t inb = nb[t];
                if (ct.count(inb)) continue;
                int n_in = countVertexInside(inb, pred);
                if (n_in == 0) { ct[inb] = ALL_OUTSIDE; continue; }
                ct[inb] = (n_in == nvc) ? (int8_t)ALL_INSIDE : centreType(inb);
                q.push_back(inb);
            }
        }
        for (int64_t c : q) {
            int8_t t = ct[c];
            if (order) order->emplace_back(c, t);
            if (t == ALL_INSIDE) inside.push_back(c); else if (t == CENTER_INSIDE) cin.push_back(c); else cout.push_back(c);
        }
        std::sort(inside.begin(), inside.end());
        std::sort(cin.begin(), cin.end());
        std::sort(cout.begin(), cout.end());
    }
    int64_t cellIndex(int64_t i, int64_t j, int64_t k) const;

    // SUBSAMPLE fraction: stratified cell-local midpoint lattice, isInside per sample (FP64)
    double subsampleFraction(int64_t c, const Solid& s) const;

    double cellFraction(int si, int64_t c, int method) override {
        const Solid& s = solids[si];
        if (method == SDFIBM_FRACTION_SUBSAMPLE) return subsampleFraction(c, s);
        Geo geo(*this);
        return geo.cellVolume(c, s, twod != 0) / vol(c);
    }

    // FP64 += that is safe when several threads add to one cell (the threaded timing variant)
    static void atomicAdd(double* a, double v) {
        uint64_t old = __atomic_load_n(reinterpret_cast<uint64_t*>(a), __ATOMIC_RELAXED), nw;
        do {
            double cur;
            std::memcpy(&cur, &old, 8);
            cur += v;
            std::memcpy(&nw, &cur, 8);
        } while (!__atomic_compare_exchange_n(reinterpret_cast<uint64_t*>(a), &old, nw, true, __ATOMIC_RELAXED,
                                              __ATOMIC_RELAXED));
    }

    // SolidCloud::solidFluidInteract (solidcloud.cpp:361-433); shared = the fields are updated by several threads
    void solidFluidInteract(int si, double dt, const double* U, double* As, double* Fs, double* Ts, int32_t* Ct,
                            int64_t N, bool shared = false) {
        Solid& s = solids[si];
        std::vector<int64_t> ins, cin, cout;
        enumerate(s, ins, cin, cout);
        size_t num_inside = ins.size();
        std::vector<int64_t> cellids;
        cellids.reserve(ins.size() + cin.size() + cout.size());
        cellids.insert(cellids.end(), ins.begin(), ins.end());
        cellids.insert(cellids.end(), cin.begin(), cin.end());
        cellids.insert(cellids.end(), cout.begin(), cout.end());
        int insideType = s.id + 4;
        for (auto c : ins) Ct[c] = insideType;
        for (auto c : cin) Ct[c] = CENTER_INSIDE;
        for (auto c : cout) Ct[c] = CENTER_OUTSIDE;
        auto& tc = touched_cells[si];
        auto& tt = touched_types[si];
        tc = cellids;
        tt.assign(cellids.size(), 0);
        for (size_t i = 0; i < cellids.size(); ++i)
            tt[i] = i < ins.size() ? ALL_INSIDE : (i < ins.size() + cin.size() ? CENTER_INSIDE : CENTER_OUTSIDE);

        Geo geo(*this);
        double dtINV = 1.0 / dt;
        V3 force{0, 0, 0}, torque{0, 0, 0};
        for (size_t counter = 0; counter < cellids.size(); ++counter) {
            int64_t c = cellids[counter];
            double alpha = num_inside > 0 ? 1.0 : 0.0;
            if (counter >= num_inside) {
                if (opt.fraction_method == SDFIBM_FRACTION_SUBSAMPLE) alpha = subsampleFraction(c, s);
                else alpha = geo.cellVolume(c, s, twod != 0) / vol(c);
            }
            if (shared) atomicAdd(As + c, alpha); else As[c] += alpha;
            V3 cc = centre(c);
            V3 uf{U[c], U[N + c], U[2 * N + c]};
            V3 us = s.evalPointVelocity(cc);
            V3 f_ = alpha * (uf - us);
            V3 t_ = cross(cc - s.center, f_);
            double cv = vol(c);
            force += f_ * cv * dtINV;
            torque += t_ * cv * dtINV;
            V3 fs = f_ * dtINV;
            if (shared) {
                atomicAdd(Fs + c, fs.x); atomicAdd(Fs + N + c, fs.y); atomicAdd(Fs + 2 * N + c, fs.z);
                atomicAdd(Ts + c, alpha);
            } else {
                Fs[c] += fs.x; Fs[N + c] += fs.y; Fs[2 * N + c] += fs.z;
                Ts[c] += alpha;
            }
        }
        force *= opt.rho_f;
        torque *= opt.rho_f;
        s.fluid_force = force;
        s.fluid_torque = torque;
    }

    // SolidCloud::interact (solidcloud.cpp:435-464).  Fields are FP64, [3][N] for vectors.
    int interact(double, double dt, const double* U, double* As, double* Fs, double* Ts, int32_t* Ct,
                 double* FT) override {
        const int64_t N = mesh.nCells();
        if (faithful || opt.dense_reset) {
            std::fill(As, As + N, 0.0); std::fill(Fs, Fs + 3 * N, 0.0);
            std::fill(Ts, Ts + N, 0.0); std::fill(Ct, Ct + N, 0);
        } else {  // sparse reset of the previous touched cells
            for (auto& v : touched_cells)
                for (int64_t c : v) { As[c] = 0; Ts[c] = 0; Ct[c] = 0; Fs[c] = Fs[N + c] = Fs[2 * N + c] = 0; }
        }
        auto t1 = std::chrono::steady_clock::now();
        for (size_t si = 0; si < solids.size(); ++si) solidFluidInteract((int)si, dt, U, As, Fs, Ts, Ct, N);
        // checkAlpha
        if (faithful || opt.dense_reset) {
            for (int64_t c = 0; c < N; ++c) As[c] = std::min(As[c], 1.0);
        } else {
            for (auto& v : touched_cells) for (int64_t c : v) As[c] = std::min(As[c], 1.0);
        }
        auto t2 = std::chrono::steady_clock::now();
        last_seconds = std::chrono::duration<double>(t2 - t1).count();
        if (FT) {
            for (size_t si = 0; si < solids.size(); ++si) {
                put3(FT + 6 * si, solids[si].fluid_force);
                put3(FT + 6 * si + 3, solids[si].fluid_torque);
            }
        }
        return 0;
    }

    // The same interact with the solids spread over nthreads host threads (solid si on thread si % nthreads), for
    // the CPU timing on all cores: as many independent solid loops as the reference would run on that many
    // single-solid-loop ranks.  Cells shared by several solids are summed atomically; Ct keeps the last writer.
    int interactThreads(double dt, const double* U, double* As, double* Fs, double* Ts, int32_t* Ct, double* FT,
                        int nthreads) override {
        const int64_t N = mesh.nCells();
        std::fill(As, As + N, 0.0); std::fill(Fs, Fs + 3 * N, 0.0);
        std::fill(Ts, Ts + N, 0.0); std::fill(Ct, Ct + N, 0);
        auto t1 = std::chrono::steady_clock::now();
        const int T = std::max(1, nthreads);
        std::vector<std::thread> pool;
        for (int t = 0; t < T; ++t)
            pool.emplace_back([&, t] {
                for (size_t si = (size_t)t; si < solids.size(); si += (size_t)T)
                    solidFluidInteract((int)si, dt, U, As, Fs, Ts, Ct, N, true);
            });
        for (auto& th : pool) th.join();
        for (int64_t c = 0; c < N; ++c) As[c] = std::min(As[c], 1.0);
        auto t2 = std::chrono::steady_clock::now();
        last_seconds = std::chrono::duration<double>(t2 - t1).count();
        if (FT) {
            for (size_t si = 0; si < solids.size(); ++si) {
                put3(FT + 6 * si, solids[si].fluid_force);
                put3(FT + 6 * si + 3, solids[si].fluid_torque);
            }
        }
        return 0;
    }

    // SolidCloud::calcMeanField<vector> for every solid (solidcloud.cpp:303-359): a copy of the solid with the sampler
    // shape (Solid::setShape keeps the pose), its cells in the enumerator's queue order, alpha = 1 inside and the
    // REF-GEO fraction on cut cells, mean = sum(alpha V U) / sum(alpha V).  Like the reference it writes Ct for every
    // cell it visits (id + 4 inside, the cell type otherwise); Ct may be NULL.
    int meanField(const sdfibm_shape_desc& sampler, const double* U, int32_t* Ct, double* out) override {
        const int64_t N = mesh.nCells();
        std::vector<int64_t> ins, cin, cout;
        std::vector<std::pair<int64_t, int8_t>> order;
        for (size_t si = 0; si < solids.size(); ++si) {
            Solid tmp = solids[si];
            tmp.d.shape = sampler;
            Geo geo(*this);
            V3 mean{0, 0, 0};
            double volume = 0.0;
            enumerate(tmp, ins, cin, cout, &order);
            const int insideType = tmp.id + 4;
            for (auto& ct : order) {
                const int64_t c = ct.first;
                double alpha;
                if (ct.second == ALL_INSIDE) {
                    alpha = 1.0;
                    if (Ct) Ct[c] = insideType;
                } else {
                    if (Ct) Ct[c] = ct.second;
                    alpha = geo.cellVolume(c, tmp, twod != 0) / vol(c);
                }
                const double dV = alpha * vol(c);
                volume += dV;
                mean += dV * V3{U[c], U[N + c], U[2 * N + c]};
            }
            put3(out + 3 * si, V3{mean.x / volume, mean.y / volume, mean.z / volume});
        }
        return 0;
    }

    int64_t touched(int si, int64_t* cells, int8_t* types, int64_t cap) const override {
        const auto& tc = touched_cells[si];
        const auto& tt = touched_types[si];
        int64_t n = (int64_t)tc.size();
        for (int64_t i = 0; i < n && i < cap; ++i) { cells[i] = tc[i]; types[i] = tt[i]; }
        return n;
    }

    // SolidCloud::fixInternal (solidcloud.cpp:288-301)
    int fixInternal(const int32_t* Ct, double* U) const override {
        const int64_t N = mesh.nCells();
        for (int64_t c = 0; c < N; ++c) {
            if (Ct[c] >= 4) {
                int id = Ct[c] - 4;
                V3 u = solids[id].evalPointVelocity(centre(c));
                U[c] = u.x; U[N + c] = u.y; U[2 * N + c] = u.z;
            }
        }
        return 0;
    }
};

// ---- UniformMesh specialisations --------------------------------------------------------------------------------
template <> V3 Cloud<UniformMesh>::point(int64_t p) const { return mesh.point(p); }
template <> int Cloud<UniformMesh>::cellPointsOf(int64_t c, int64_t* out) const { mesh.cellPoints(c, out); return 8; }
template <> int Cloud<UniformMesh>::cellFacesOf(int64_t c, FaceRef* out) const { return mesh.cellFaces(c, out); }
template <> int Cloud<UniformMesh>::cellCellsOf(int64_t c, int64_t* out) const { return mesh.cellCells(c, out); }
template <> V3 Cloud<UniformMesh>::centre(int64_t c) const { return mesh.C(c); }
template <> double Cloud<UniformMesh>::vol(int64_t c) const { return mesh.V(c); }
template <> int64_t Cloud<UniformMesh>::cellIndex(int64_t i, int64_t j, int64_t k) const { return mesh.cell(i, j, k); }

template <> template <class Pred>
int Cloud<UniformMesh>::countVertexInside(int64_t c, const Pred& pred) const {
    int64_t v[8];
    mesh.cellPoints(c, v);
    int n = 0;
    for (int i = 0; i < 8; ++i) n += pred(mesh.point(v[i]));
    return n;
}

template <> int64_t Cloud<UniformMesh>::findNearestCell(const V3& p) const {
    if (faithful) {
        int64_t best = 0;
        double bd = magSqr(mesh.C(0) - p);
        for (int64_t c = 1; c < mesh.nCells(); ++c) {
            double d = magSqr(mesh.C(c) - p);
            if (d < bd) { bd = d; best = c; }
        }
        return best;
    }
    const double* o = mesh.d.origin; const double* h = mesh.d.h;
    int64_t n[3] = {mesh.nx, mesh.ny, mesh.nz};
    double pc[3] = {p.x, p.y, p.z};
    int64_t lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
        double t = std::floor((pc[a] - o[a]) / h[a]);
        int64_t e = !(t >= 0) ? 0 : (t > (double)(n[a] - 1) ? n[a] - 1 : (int64_t)t);  // NaN: 0, as the device
        lo[a] = std::max<int64_t>(0, e - 1); hi[a] = std::min<int64_t>(n[a] - 1, e + 1);
    }
    int64_t best = -1;
    double bd = 0;
    for (int64_t k = lo[2]; k <= hi[2]; ++k)
        for (int64_t j = lo[1]; j <= hi[1]; ++j)
            for (int64_t i = lo[0]; i <= hi[0]; ++i) {
                int64_t c = mesh.cell(i, j, k);
                double d = magSqr(mesh.C(c) - p);
                if (best < 0 || d < bd || (d == bd && c < best)) { bd = d; best = c; }
            }
    return best;
}

// Conservative radius of the region where isInside can be true, measured from the shape's local origin shifted by
// -com.  (IShape::m_radiusB is not a bound for Rectangle, Box and the tails, so it is not used here.)
static bool shapeBoundRadius(const sdfibm_shape_desc& s, double& r, bool& prism) {
    const double* a = s.p;
    prism = false;
    switch (s.type) {
        case SDFIBM_SHAPE_CIRCLE: r = a[0]; prism = true; return true;
        case SDFIBM_SHAPE_SPHERE: r = a[0]; return true;
        case SDFIBM_SHAPE_ELLIPSE: r = std::max(a[0], a[1]); prism = true; return true;
        case SDFIBM_SHAPE_ELLIPSOID: r = std::max({a[0], a[1], a[2]}); return true;
        case SDFIBM_SHAPE_RECTANGLE: r = std::sqrt(a[0] * a[0] + a[1] * a[1]); prism = true; return true;
        case SDFIBM_SHAPE_BOX: r = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); return true;
        case SDFIBM_SHAPE_CIRCLE_TAIL:
        case SDFIBM_SHAPE_CIRCLE_TWOTAIL:
            r = std::max(a[0], std::sqrt(4 * a[4] * a[4] + a[2] * a[2])); prism = true; return true;
        default: return false;
    }
}

template <> bool Cloud<UniformMesh>::bboxCells(const Solid& s, int64_t lo[3], int64_t hi[3]) const {
    double r;
    bool prism;
    if (!shapeBoundRadius(s.d.shape, r, prism)) return false;
    const double* com = s.d.shape.com;
    // the inside region is centred at -com in the local frame (Ellipsoid ignores com)
    V3 cl{-com[0], -com[1], -com[2]};
    if (s.d.shape.type == SDFIBM_SHAPE_ELLIPSOID) cl = V3{0, 0, 0};
    if (prism) {
        // a 2-D shape is a prism along local z; bounded in world only when local z stays world z
        if (!(s.q.v.x == 0.0 && s.q.v.y == 0.0)) return false;
        cl.z = 0.0;
    }
    V3 cw = s.center + transform(s.q, cl);
    r = r * (1.0 + 1e-9) + 1e-12;
    int64_t n[3] = {mesh.nx, mesh.ny, mesh.nz};
    double c3[3] = {cw.x, cw.y, cw.z};
    for (int a = 0; a < 3; ++a) {
        if (prism && a == 2) { lo[a] = 0; hi[a] = n[a] - 1; continue; }
        double l = std::floor((c3[a] - r - mesh.d.origin[a]) / mesh.d.h[a]) - 1;
        double u = std::floor((c3[a] + r - mesh.d.origin[a]) / mesh.d.h[a]) + 1;
        lo[a] = (int64_t)std::min(std::max(0.0, l), (double)n[a]);
        hi[a] = (int64_t)std::max(std::min((double)(n[a] - 1), u), -1.0);
    }
    return true;
}

template <> double Cloud<UniformMesh>::subsampleFraction(int64_t c, const Solid& s) const {
    int n = opt.subsample_n > 0 ? opt.subsample_n : 10;
    int64_t i, j, k;
    mesh.ijk(c, i, j, k);
    const double* o = mesh.d.origin; const double* h = mesh.d.h;
    int nzs = twod ? 1 : n;
    int64_t cnt = 0;
    for (int c3 = 0; c3 < nzs; ++c3) {
        double tz = twod ? 0.5 : (double)(2 * c3 + 1) / (double)(2 * n);
        double z = o[2] + ((double)k + tz) * h[2];
        for (int b = 0; b < n; ++b) {
            double y = o[1] + ((double)j + (double)(2 * b + 1) / (double)(2 * n)) * h[1];
            for (int a = 0; a < n; ++a) {
                double x = o[0] + ((double)i + (double)(2 * a + 1) / (double)(2 * n)) * h[0];
                cnt += s.phi01(V3{x, y, z});
            }
        }
    }
    return (double)cnt / (double)(n * n * nzs);
}

// ---- PolyMesh specialisations -----------------------------------------------------------------------------------
template <> V3 Cloud<PolyMesh>::point(int64_t p) const { return mesh.points[p]; }
template <> int Cloud<PolyMesh>::cellPointsOf(int64_t c, int64_t* out) const {
    const auto& v = mesh.cellPointsL[c];
    int n = (int)std::min<size_t>(8, v.size());
    for (int i = 0; i < n; ++i) out[i] = v[i];
    return n;
}
template <> int Cloud<PolyMesh>::cellFacesOf(int64_t c, FaceRef* out) const {
    const auto& fl = mesh.cells[c];
    int n = (int)std::min<size_t>(12, fl.size());
    for (int q = 0; q < n; ++q) {
        const auto& fv = mesh.faces[fl[q]];
        for (int t = 0; t < 4; ++t) out[q].v[t] = fv[t];
        out[q].Cf = mesh.Cf[fl[q]]; out[q].Sf = mesh.Sf[fl[q]];
    }
    return n;
}
template <> int Cloud<PolyMesh>::cellCellsOf(int64_t c, int64_t* out) const {
    const auto& v = mesh.cellCellsL[c];
    int n = (int)std::min<size_t>(6, v.size());
    for (int i = 0; i < n; ++i) out[i] = v[i];
    return n;
}
template <> V3 Cloud<PolyMesh>::centre(int64_t c) const { return mesh.Cc[c]; }
template <> double Cloud<PolyMesh>::vol(int64_t c) const { return mesh.Vc[c]; }
template <> int64_t Cloud<PolyMesh>::cellIndex(int64_t, int64_t, int64_t) const { return -1; }
template <> template <class Pred>
int Cloud<PolyMesh>::countVertexInside(int64_t c, const Pred& pred) const {
    int n = 0;
    for (int64_t p : mesh.cellPointsL[c]) n += pred(mesh.points[p]);
    return n;
}
template <> int64_t Cloud<PolyMesh>::findNearestCell(const V3& p) const {
    int64_t best = 0;
    double bd = magSqr(mesh.Cc[0] - p);
    for (int64_t c = 1; c < mesh.nCells(); ++c) {
        double d = magSqr(mesh.Cc[c] - p);
        if (d < bd) { bd = d; best = c; }
    }
    return best;
}
template <> bool Cloud<PolyMesh>::bboxCells(const Solid&, int64_t*, int64_t*) const { return false; }
template <> double Cloud<PolyMesh>::subsampleFraction(int64_t, const Solid&) const { return 0.0; }

}  // namespace oracle

using namespace oracle;

// ---- C interface (ctypes) ---------------------------------------------------------------------------------------
extern "C" {

int oracle_abi_version(void) { return SDFIBM_ABI_VERSION; }

void* oracle_create_uniform(const sdfibm_mesh_desc* mesh, const sdfibm_solid_desc* solids, int n,
                            const sdfibm_options* opt, int faithful) {
    try {
        auto m = std::make_unique<UniformMesh>(*mesh);
        auto* c = new Cloud<UniformMesh>(std::move(m), solids, n, *opt, faithful != 0);
        c->twod = mesh->twod;
        c->bmin = c->mesh.boundsMin(); c->bmax = c->mesh.boundsMax();
        return c;
    } catch (...) { return nullptr; }
}

// points: [npoints][3]; face_off: nfaces+1; face_lab; owner: nfaces; neighbour: ninternal
void* oracle_create_polymesh(const double* points, int64_t npoints, const int32_t* face_off, const int32_t* face_lab,
                             int64_t nfaces, const int32_t* owner, const int32_t* neighbour, int64_t ninternal,
                             int twod, const sdfibm_solid_desc* solids, int n, const sdfibm_options* opt) {
    try {
        auto m = std::make_unique<PolyMesh>();
        m->points.resize(npoints);
        for (int64_t p = 0; p < npoints; ++p) m->points[p] = V3{points[3 * p], points[3 * p + 1], points[3 * p + 2]};
        m->faces.resize(nfaces);
        for (int64_t f = 0; f < nfaces; ++f)
            for (int32_t q = face_off[f]; q < face_off[f + 1]; ++q) m->faces[f].push_back(face_lab[q]);
        m->owner.assign(owner, owner + nfaces);
        m->neighbour.assign(neighbour, neighbour + ninternal);
        m->build();
        auto* c = new Cloud<PolyMesh>(std::move(m), solids, n, *opt, true);
        c->twod = twod;
        c->bmin = c->mesh.bmin; c->bmax = c->mesh.bmax;
        return c;
    } catch (...) { return nullptr; }
}

void oracle_destroy(void* h) { delete static_cast<CloudBase*>(h); }
int64_t oracle_ncells(void* h) { return static_cast<CloudBase*>(h)->nCells(); }

int oracle_interact(void* h, double time, double dt, const double* U, double* As, double* Fs, double* Ts, int32_t* Ct,
                    double* FT) {
    try { return static_cast<CloudBase*>(h)->interact(time, dt, U, As, Fs, Ts, Ct, FT); } catch (...) { return 1; }
}
double oracle_last_seconds(void* h) { return static_cast<CloudBase*>(h)->last_seconds; }
int oracle_interact_threads(void* h, double dt, const double* U, double* As, double* Fs, double* Ts, int32_t* Ct,
                            double* FT, int nthreads) {
    return static_cast<CloudBase*>(h)->interactThreads(dt, U, As, Fs, Ts, Ct, FT, nthreads);
}
int64_t oracle_last_pairs(void* h) { return static_cast<CloudBase*>(h)->last_pairs; }

int oracle_mean_field(void* h, const sdfibm_shape_desc* sampler, const double* U, int32_t* Ct, double* out) {
    return static_cast<CloudBase*>(h)->meanField(*sampler, U, Ct, out);
}
int64_t oracle_touched(void* h, int s, int64_t* cells, int8_t* types, int64_t cap) {
    return static_cast<CloudBase*>(h)->touched(s, cells, types, cap);
}
int oracle_evolve(void* h, double time, double dt) { return static_cast<CloudBase*>(h)->evolve(time, dt); }
int oracle_fix_internal(void* h, const int32_t* Ct, double* U) { return static_cast<CloudBase*>(h)->fixInternal(Ct, U); }
int oracle_get_state(void* h, sdfibm_solid_state* out, int n) {
    auto* c = static_cast<CloudBase*>(h);
    for (int i = 0; i < n && i < (int)c->solids.size(); ++i) c->getState(i, out[i]);
    return 0;
}
int oracle_set_state(void* h, const sdfibm_solid_state* in, int n) {
    auto* c = static_cast<CloudBase*>(h);
    for (int i = 0; i < n && i < (int)c->solids.size(); ++i) c->setState(i, in[i]);
    return 0;
}
void oracle_cell_centre(void* h, int64_t c, double* out) { static_cast<CloudBase*>(h)->cellCentre(c, out); }
double oracle_cell_fraction(void* h, int s, int64_t c, int method) {
    return static_cast<CloudBase*>(h)->cellFraction(s, c, method);
}

// Shape constructor restatement (for checking the host-side lowering)
int oracle_make_shape(int type, const double* raw, const double* com, sdfibm_shape_desc* out) {
    try { *out = makeShape(type, raw, com); return 0; } catch (...) { return 1; }
}
// quaternion(XYZ, euler in radians) and Solid::setMaterial
void oracle_quat_from_euler(const double* angles, double* q4) {
    Quat q = fromEulerXYZ(V3{angles[0], angles[1], angles[2]});
    q4[0] = q.w; q4[1] = q.v.x; q4[2] = q.v.y; q4[3] = q.v.z;
}
void oracle_world2local(const double* p, const double* t, const double* q4, double* out) {
    V3 r = world2local(arr3(p), arr3(t), Quat{q4[0], arr3(q4 + 1)});
    put3(out, r);
}
int oracle_phi01(const sdfibm_solid_desc* s, const double* p) {
    return shapeInside(s->shape, world2local(arr3(p), arr3(s->pos), Quat{s->quat[0], arr3(s->quat + 1)}));
}
double oracle_phi(const sdfibm_solid_desc* s, const double* p) {
    return shapeSDF(s->shape, world2local(arr3(p), arr3(s->pos), Quat{s->quat[0], arr3(s->quat + 1)}));
}

// One labelled training cell of the learned fraction (sdfibm_mlp_dataset): the shape at the origin with rotation q4,
// the cell [o, o + h]^3; writes the signed distance divided by h at the 5 x 5 x 5 lattice of the cell (spacing h/4,
// index i + 5 (j + 5 k)) and returns the number of n^3 midpoint-lattice samples inside.
int64_t oracle_sample_cell(const sdfibm_shape_desc* s, const double* q4, const double* o, double h, int n,
                           double* phi125) {
    const Quat q{q4[0], V3{q4[1], q4[2], q4[3]}};
    const V3 zero{0.0, 0.0, 0.0};
    for (int k = 0; k < 5; ++k)
        for (int j = 0; j < 5; ++j)
            for (int i = 0; i < 5; ++i) {
                const V3 p{o[0] + 0.25 * i * h, o[1] + 0.25 * j * h, o[2] + 0.25 * k * h};
                phi125[i + 5 * (j + 5 * k)] = shapeSDF(*s, world2local(p, zero, q)) / h;
            }
    int64_t cnt = 0;
    for (int c = 0; c < n; ++c)
        for (int b = 0; b < n; ++b)
            for (int a = 0; a < n; ++a) {
                const double ta = (double)(2 * a + 1) / (double)(2 * n), tb = (double)(2 * b + 1) / (double)(2 * n),
                             tc = (double)(2 * c + 1) / (double)(2 * n);
                const V3 p{o[0] + ta * h, o[1] + tb * h, o[2] + tc * h};
                cnt += shapeInside(*s, world2local(p, zero, q)) ? 1 : 0;
            }
    return cnt;
}

}  // extern "C"
