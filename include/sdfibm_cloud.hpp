/*
 * sdfibm_cloud.hpp -- the reference's SolidCloud interface (src/solidcloud.h:89-124) in C++17 over the C ABI of
 * sdfibm_cuda.h and sdfibm_host.h, for callers that keep their fields in host memory (header only; link
 * libsdfibm_cuda.so).  Same method names and meaning as the reference:
 *
 *   SolidCloud(dict_text, mesh, rho_f, time)   SolidCloud::SolidCloud + initFromDictionary (initialCorrect at t = 0)
 *   interact(time, dt)                         SolidCloud::interact: As, Fs, Ts, Ct and each solid's fluid force
 *   evolve(time, dt)                           SolidCloud::evolve
 *   fixInternal(dt)                            SolidCloud::fixInternal: U = the owner's rigid velocity where Ct >= 4
 *   saveState()                                cloud.out every writeFrequency calls, meanfield.out on every call
 *   saveRestart(filename)                      the solidDict with the current pos, vel, euler, omega
 *   writeMeanField(), totalSolidVolume(), operator[](i), isOnFluid(), isOnTwoD()
 *
 * Fields are cell-major float arrays: U and Fs as x, y, z planes of N cells, As and Ts of N, Ct int32 of N.  The
 * caller writes U() before interact and reads the others after it.  Errors throw std::runtime_error with the
 * library's message (the reference quits the process instead).
 */
#ifndef SDFIBM_CLOUD_HPP
#define SDFIBM_CLOUD_HPP

#include <cstdint>
#include <cstdio>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "sdfibm_cuda.h"
#include "sdfibm_host.h"

namespace sdfibm_gb300 {

class SolidCloud {
public:
    /* dict_text: the solidDict; mesh: the uniform mesh (twod is taken from meta.on_twod); rho_f: the
     * transportProperties density (0 is used when meta.on_fluid is off); time: the start time, initialCorrect runs
     * when it is 0 (src/solidcloud.cpp:252-258), on U0 (3 N floats; NULL: U = 0); state_path: cloud.out (""
     * writes none; meanfield.out, when meta.on_meanfield is present, goes to the working directory as in the
     * reference); opt: options of the GPU path (NULL: the library's defaults), gravity and rho_f always come from
     * the dictionary. */
    SolidCloud(const std::string& dict_text, const sdfibm_mesh_desc& mesh, double rho_f, double time,
               const float* U0 = nullptr, const std::string& state_path = "cloud.out",
               const sdfibm_options* opt = nullptr)
        : dict_(dict_text), mesh_(mesh), time_(time) {
        char msg[512] = {0};
        int32_t n = 0, twod = 0;
        sdfibm_options parsed;
        if (sdfibm_host_parse_soliddict(dict_.c_str(), rho_f, nullptr, 0, &n, &parsed, &twod, msg, sizeof msg) !=
                SDFIBM_OK &&
            n == 0)
            throw std::runtime_error(std::string("solidDict: ") + msg);
        solids_.resize((size_t)(n > 0 ? n : 1));
        if (sdfibm_host_parse_soliddict(dict_.c_str(), rho_f, solids_.data(), n, &n, &parsed, &twod, msg,
                                        sizeof msg) != SDFIBM_OK)
            throw std::runtime_error(std::string("solidDict: ") + msg);
        solids_.resize((size_t)n);
        opt_ = parsed;
        if (opt) {
            opt_ = *opt;
            opt_.rho_f = parsed.rho_f;
            for (int a = 0; a < 3; ++a) opt_.gravity[a] = parsed.gravity[a];
        }
        mesh_.twod = twod;
        N_ = (int64_t)mesh_.nx * mesh_.ny * mesh_.nz;
        write_frequency_ = std::stoi(lookup("meta/writeFrequency", "1"));
        if (write_frequency_ < 1) throw std::runtime_error("meta.writeFrequency must be positive");
        const std::string sampler = lookup("meta/sampler", "");
        on_meanfield_ = lookup("meta/on_meanfield", "\x01") != "\x01";  // meta.found("on_meanfield")
        const std::string fl = lookup("meta/on_fluid", "0");                // Foam::readBool
        on_fluid_ = fl == "1" || fl == "true" || fl == "yes" || fl == "on" || fl == "y" || fl == "t";
        if (!sampler.empty()) {
            if (sdfibm_host_soliddict_shape(dict_.c_str(), sampler.c_str(), &sampler_shape_, msg, sizeof msg) !=
                SDFIBM_OK)
                throw std::runtime_error(std::string("sampler: ") + msg);
            has_sampler_ = true;
        }
        check(sdfibm_cuda_create(&mesh_, solids_.data(), (int32_t)solids_.size(), &opt_, nullptr, &ctx_), "create");
        U_.assign((size_t)(3 * N_), 0.0f);
        if (U0) U_.assign(U0, U0 + 3 * N_);
        As_.assign((size_t)N_, 0.0f);
        Fs_.assign((size_t)(3 * N_), 0.0f);
        Ts_.assign((size_t)N_, 0.0f);
        Ct_.assign((size_t)N_, 0);
        FT_.assign(6 * solids_.size() + 6, 0.0);
        if (!state_path.empty()) {
            statefile_.open(state_path, std::ios::out | std::ios::trunc);
            if (!statefile_) throw std::runtime_error("cannot open " + state_path);
        }
        if (on_meanfield_) meanfile_.open("meanfield.out", std::ios::out | std::ios::trunc);
        if (!(time > 0)) initialCorrect();
    }
    ~SolidCloud() {
        if (sampler_ctx_) sdfibm_cuda_destroy(sampler_ctx_);
        if (ctx_) sdfibm_cuda_destroy(ctx_);
    }
    SolidCloud(const SolidCloud&) = delete;
    SolidCloud& operator=(const SolidCloud&) = delete;

    std::vector<float>& U() { return U_; }
    const std::vector<float>& As() const { return As_; }
    const std::vector<float>& Fs() const { return Fs_; }
    const std::vector<float>& Ts() const { return Ts_; }
    const std::vector<int32_t>& Ct() const { return Ct_; }
    /* force (3) and torque (3) on each solid from the last interact */
    const double* fluidForceTorque(int i) const { return FT_.data() + 6 * i; }
    int size() const { return (int)solids_.size(); }
    double time() const { return time_; }

    void interact(double time, double dt) {
        check(sdfibm_cuda_interact_host(ctx_, time, dt, U_.data(), As_.data(), Fs_.data(), Ts_.data(), Ct_.data(),
                                        FT_.data()),
              "interact");
    }

    void evolve(double time, double dt) {
        check(sdfibm_cuda_evolve(ctx_, time, dt), "evolve");
        time_ = time;
    }

    /* src/solidcloud.cpp:288-301 over the host fields: every cell with Ct >= 4 (the coupling's inside cells, and the
     * sampler's after writeMeanField, as in the reference) takes its solid's velocity at the cell centre */
    void fixInternal(double /*dt*/) {
        const std::vector<sdfibm_solid_state> st = states();
        for (int64_t c = 0; c < N_; ++c) {
            const int32_t ct = Ct_[(size_t)c];
            if (ct < 4) continue;
            const size_t id = (size_t)(ct - 4);
            if (id >= st.size()) continue;
            const int64_t i = c % mesh_.nx, j = (c / mesh_.nx) % mesh_.ny, k = c / ((int64_t)mesh_.nx * mesh_.ny);
            const double cc[3] = {mesh_.origin[0] + ((double)i + 0.5) * mesh_.h[0],
                                  mesh_.origin[1] + ((double)j + 0.5) * mesh_.h[1],
                                  mesh_.origin[2] + ((double)k + 0.5) * mesh_.h[2]};
            const sdfibm_solid_state& s = st[id];
            const double r[3] = {cc[0] - s.pos[0], cc[1] - s.pos[1], cc[2] - s.pos[2]};
            const double u[3] = {s.vel[0] + (s.omega[1] * r[2] - s.omega[2] * r[1]),
                                 s.vel[1] + (s.omega[2] * r[0] - s.omega[0] * r[2]),
                                 s.vel[2] + (s.omega[0] * r[1] - s.omega[1] * r[0])};
            for (int a = 0; a < 3; ++a) U_[(size_t)(a * N_ + c)] = (float)u[a];
        }
    }

    /* src/solidcloud.cpp:276-286 */
    void initialCorrect() {
        interact(0.0, 1.0);
        std::vector<sdfibm_solid_state> st = states();
        for (auto& s : st)
            for (int a = 0; a < 3; ++a) s.force[a] = s.torque[a] = 0.0;
        check(sdfibm_cuda_set_solids(ctx_, st.data(), (int32_t)st.size()), "set_solids");
    }

    /* src/solidcloud.cpp:578-593 */
    void saveState() {
        if (counter_ % (unsigned)write_frequency_ == 0 && statefile_.is_open()) {
            const std::vector<sdfibm_solid_state> st = states();
            statefile_ << text([&](char* b, int64_t cap, int64_t* len) {
                return sdfibm_host_format_state(time_, mesh_.twod, st.data(), (int32_t)st.size(), b, cap, len);
            });
            statefile_.flush();
        }
        if (on_meanfield_) writeMeanField();
        ++counter_;
    }

    /* src/solidcloud.cpp:616-665 */
    void saveRestart(const std::string& filename, int precision = 6) const {
        const std::vector<sdfibm_solid_state> st = states();
        char msg[512] = {0};
        int64_t len = 0;
        check_host(sdfibm_host_write_restart(dict_.c_str(), st.data(), (int32_t)st.size(), mesh_.twod, precision,
                                             nullptr, nullptr, 0, &len, msg, sizeof msg),
                   msg);
        std::string out((size_t)len + 1, '\0');
        check_host(sdfibm_host_write_restart(dict_.c_str(), st.data(), (int32_t)st.size(), mesh_.twod, precision,
                                             nullptr, &out[0], len + 1, &len, msg, sizeof msg),
                   msg);
        out.resize((size_t)len);
        std::ofstream os(filename, std::ios::out | std::ios::trunc);
        if (!os) throw std::runtime_error("cannot open " + filename);
        os << out;
    }

    /* src/solidcloud.cpp:303-359: the mean of U over each solid's sampler shape; it also writes Ct on the cells a
     * sampler visits, as the reference does.  The means come from two coupling passes of the sampler-shaped solids
     * at rest with rho_f = 1 and dt = 1 (sum(alpha V U), then sum(alpha V) on U = 1). */
    void writeMeanField() {
        if (!has_sampler_) return;
        const std::vector<double> m = meanField();
        if (meanfile_.is_open()) {
            meanfile_ << text([&](char* b, int64_t cap, int64_t* len) {
                return sdfibm_host_format_mean_field(m.data(), (int32_t)(m.size() / 3), b, cap, len);
            });
            meanfile_.flush();
        }
    }

    std::vector<double> meanField() {
        if (!has_sampler_) throw std::runtime_error("meanField needs meta.sampler");
        if (!sampler_ctx_) {
            std::vector<sdfibm_solid_desc> ss = solids_;
            for (auto& d : ss) d.shape = sampler_shape_;
            sdfibm_options o;
            sdfibm_options_default(&o);
            o.rho_f = 1.0;
            o.fraction_method = SDFIBM_FRACTION_REFGEO;
            o.exact_forcing = 1;
            check(sdfibm_cuda_create(&mesh_, ss.data(), (int32_t)ss.size(), &o, nullptr, &sampler_ctx_), "create",
                  sampler_ctx_);
            sAs_.assign((size_t)N_, 0.0f);
            sFs_.assign((size_t)(3 * N_), 0.0f);
            sTs_.assign((size_t)N_, 0.0f);
            sCt_.assign((size_t)N_, 0);
            ones_.assign((size_t)(3 * N_), 1.0f);
        }
        std::vector<sdfibm_solid_state> st = states();
        for (auto& s : st)
            for (int a = 0; a < 3; ++a) s.vel[a] = s.omega[a] = 0.0;
        check(sdfibm_cuda_set_solids(sampler_ctx_, st.data(), (int32_t)st.size()), "set_solids", sampler_ctx_);
        std::vector<double> F(6 * st.size() + 6), W(6 * st.size() + 6);
        check(sdfibm_cuda_interact_host(sampler_ctx_, time_, 1.0, U_.data(), sAs_.data(), sFs_.data(), sTs_.data(),
                                        sCt_.data(), F.data()),
              "interact", sampler_ctx_);
        check(sdfibm_cuda_interact_host(sampler_ctx_, time_, 1.0, ones_.data(), sAs_.data(), sFs_.data(),
                                        sTs_.data(), sCt_.data(), W.data()),
              "interact", sampler_ctx_);
        for (int64_t c = 0; c < N_; ++c)
            if (sCt_[(size_t)c] != 0) Ct_[(size_t)c] = sCt_[(size_t)c];
        std::vector<double> m(3 * st.size());
        for (size_t i = 0; i < st.size(); ++i)
            for (int a = 0; a < 3; ++a) m[3 * i + a] = F[6 * i + a] / W[6 * i];
        return m;
    }

    /* src/solidcloud.cpp:572-576 */
    double totalSolidVolume() const {
        double s = 0.0;
        for (float a : As_) s += a;
        return s * mesh_.h[0] * mesh_.h[1] * mesh_.h[2];
    }

    sdfibm_solid_state operator[](int i) const {
        if (i < 0 || i >= size()) throw std::out_of_range("solid index");
        return states()[(size_t)i];
    }
    bool isOnFluid() const { return on_fluid_; }
    bool isOnTwoD() const { return mesh_.twod != 0; }

    std::vector<sdfibm_solid_state> states() const {
        std::vector<sdfibm_solid_state> st(solids_.size());
        if (!st.empty()) check(sdfibm_cuda_get_solids(ctx_, st.data(), (int32_t)st.size()), "get_solids");
        return st;
    }
    sdfibm_ctx* context() const { return ctx_; }

private:
    void check(int rc, const char* what, const sdfibm_ctx* on = nullptr) const {
        if (rc == SDFIBM_OK) return;
        const sdfibm_ctx* c = on ? on : ctx_;
        throw std::runtime_error(std::string(what) + ": " + (c ? sdfibm_cuda_last_error(c) : "failed"));
    }
    static void check_host(int rc, const char* msg) {
        if (rc != SDFIBM_OK) throw std::runtime_error(msg);
    }
    template <class F> static std::string text(F&& call) {
        int64_t len = 0;
        check_host(call(nullptr, 0, &len), "text output");
        std::string out((size_t)len + 1, '\0');
        check_host(call(&out[0], len + 1, &len), "text output");
        out.resize((size_t)len);
        return out;
    }
    std::string lookup(const char* path, const std::string& dflt) const {
        int64_t len = 0;
        if (sdfibm_host_soliddict_lookup(dict_.c_str(), path, nullptr, 0, &len) != SDFIBM_OK || len < 0) return dflt;
        std::string out((size_t)len + 1, '\0');
        sdfibm_host_soliddict_lookup(dict_.c_str(), path, &out[0], len + 1, &len);
        out.resize((size_t)len);
        return out;
    }

    std::string dict_;
    sdfibm_mesh_desc mesh_;
    sdfibm_options opt_{};
    std::vector<sdfibm_solid_desc> solids_;
    sdfibm_ctx* ctx_ = nullptr;
    sdfibm_ctx* sampler_ctx_ = nullptr;
    sdfibm_shape_desc sampler_shape_{};
    bool has_sampler_ = false, on_meanfield_ = false, on_fluid_ = false;
    int write_frequency_ = 1;
    unsigned counter_ = 0;
    double time_ = 0.0;
    int64_t N_ = 0;
    std::vector<float> U_, As_, Fs_, Ts_, sAs_, sFs_, sTs_, ones_;
    std::vector<int32_t> Ct_, sCt_;
    std::vector<double> FT_;
    std::ofstream statefile_, meanfile_;
};

}  // namespace sdfibm_gb300

#endif /* SDFIBM_CLOUD_HPP */
