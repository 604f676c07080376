// CCUDAParticleSimulator.hpp -- Qt-free C++ mirror of the reference's simulator interface
// (CBaseParticleSimulator, include/CBaseParticleSimulator.h:29-110) for the CUDA step.
//
// Same method names and meaning as the reference: the constructor takes the cubic box size
// and the scenario; setupScene() adds the scenario's particles
// (src/CBaseParticleSimulator.cpp:38-65); step() runs generateParticles and the five passes in
// the reference's order (:116-144); the pass methods return milliseconds (0 when profiling is
// off, and 0 for updateCollisions/integrate, which are fused into updateForces); a failing
// step stops the simulator and reports through the errorOccured callback, as
// CGPUBaseParticleSimulator::step does (src/CGPUBaseParticleSimulator.cpp:28-37). A Qt
// subclass of CBaseParticleSimulator makes the same calls in the same order.
#ifndef CCUDAPARTICLESIMULATOR_HPP
#define CCUDAPARTICLESIMULATOR_HPP

#include <chrono>
#include <cmath>
#include <cstdio>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "sph_cuda.h"

enum SimulationScenario { DAM_BREAK = 0, FOUNTAIN };  // include/CBaseParticleSimulator.h:21-25

// One step's pass times in ms and the frame rate (include/SProfilingEvent.h:7-31).
struct sProfilingEvent {
    unsigned long iteration;
    double fps = 0, updateGrid = 0, updateDensityPressure = 0, updateForces = 0, updateCollisions = 0, integrate = 0;
    explicit sProfilingEvent(unsigned long it) : iteration(it) {}
    double together() const { return updateGrid + updateDensityPressure + updateForces + updateCollisions + integrate; }
};

class CCUDAParticleSimulator
{
public:
    struct SphException : std::runtime_error {
        int code;
        SphException(int c, const std::string &m) : std::runtime_error(m), code(c) {}
    };

    explicit CCUDAParticleSimulator(float boxSize, SimulationScenario scenario = DAM_BREAK, bool profiling = true,
                                    int precision = SPH_PLAIN_F32)
        : m_boxSize(boxSize), m_scenario(scenario), m_profiling(profiling), m_precision(precision)
    {
        m_gravity[0] = 0.0f;
        m_gravity[1] = -9.80665f;  // GRAVITY_ACCELERATION, include/CBaseParticleSimulator.h:19
        m_gravity[2] = 0.0f;
    }
    ~CCUDAParticleSimulator() { sph_destroy(m_ctx); }
    CCUDAParticleSimulator(const CCUDAParticleSimulator &) = delete;
    CCUDAParticleSimulator &operator=(const CCUDAParticleSimulator &) = delete;

    std::function<void(const char *)> errorOccured;  // the errorOccured(const char*) signal

    void setupScene()
    {
        const double halfParticle = 0.0457f / 2.0f;
        const unsigned calculatedCount = (unsigned) (std::ceil(m_boxSize / halfParticle) *
                                                     std::ceil(m_boxSize / halfParticle) *
                                                     std::ceil(m_boxSize / 4 / halfParticle));
        std::vector<float> xyz;
        if (m_scenario == DAM_BREAK) {
            const int64_t n = sph_scene_reference_dam_break(m_boxSize, nullptr, 0);
            xyz.resize(3 * (size_t) n);
            sph_scene_reference_dam_break(m_boxSize, xyz.data(), (uint64_t) n);
            if ((unsigned) n != calculatedCount) throw SphException(SPH_ERR_STATE, "scene count mismatch");
            m_maxParticlesCount = (unsigned) n;
        } else {
            m_maxParticlesCount = calculatedCount;
        }
        sph_params p;
        sph_params_default(&p);
        for (int a = 0; a < 3; a++) p.gravity[a] = m_gravity[a];
        p.flags = m_profiling ? SPH_FLAG_PROFILE : 0u;
        p.precision = m_precision;
        const float box[3] = {m_boxSize, m_boxSize, m_boxSize};
        sph_destroy(m_ctx);
        m_ctx = nullptr;
        check(sph_create(&p, box, m_maxParticlesCount ? m_maxParticlesCount : 1, &m_ctx), true);
        const uint32_t count = (uint32_t) (xyz.size() / 3);
        check(sph_upload(m_ctx, xyz.data(), nullptr, &count));
        m_particlesCount = count;
    }

    void setGravityVector(const float g[3])
    {
        for (int a = 0; a < 3; a++) m_gravity[a] = g[a];
        if (m_ctx) check(sph_set_gravity(m_ctx, -1, m_gravity));
    }

    std::string getSelectedDevice() const { return m_ctx ? sph_device_name(m_ctx) : std::string(); }

    void step()
    {
        try {
            generateParticles();
            m_last[0] = updateGrid();
            m_last[1] = updateDensityPressure();
            m_last[2] = updateForces();
            m_last[3] = updateCollisions();
            m_last[4] = integrate();
            if (m_profiling && m_totalIteration % eventLoggerStride == 0) {  // src/CBaseParticleSimulator.cpp:138-142
                sProfilingEvent e(m_totalIteration);
                e.fps = getFps();
                e.updateGrid = m_last[0];
                e.updateDensityPressure = m_last[1];
                e.updateForces = m_last[2];
                e.updateCollisions = m_last[3];
                e.integrate = m_last[4];
                events.push_back(e);
            }
            ++m_totalIteration;
            ++m_iterationSincePaused;
        } catch (const SphException &e) {
            if (errorOccured) errorOccured(e.what());
            stop();
        }
    }

    void start()
    {
        m_running = true;
        m_iterationSincePaused = 0;
        m_t0 = std::chrono::steady_clock::now();
    }
    void stop() { m_running = false; }
    bool isRunning() const { return m_running; }

    unsigned long getParticlesCount() const { return m_particlesCount; }
    unsigned long getMaxParticlesCount() const { return m_maxParticlesCount; }
    unsigned long getTotalIteration() const { return m_totalIteration; }
    const double *lastPassTimes() const { return m_last; }  // grid, density, forces, collisions, integrate
    sph_ctx *context() { return m_ctx; }

    // profiling log (include/CBaseParticleSimulator.h:54-55)
    std::vector<sProfilingEvent> events;
    int eventLoggerStride = 10;

    // steps per second since the simulation was last started (CBaseParticleSimulator::getFps)
    double getFps() const
    {
        const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - m_t0).count();
        return el > 0 ? m_iterationSincePaused / el : 0.0;
    }

    // Appends the two profiling logs of MainWindow::exportLogs (src/mainwindow.cpp:310-368) to
    // <dir>/<scenario>_<box>.csv (one "type;together;...;" line) and <dir>/<scenario>_<box>_detail.csv
    // (the type, one "label;v;...;" line per pass, two blank lines). Numbers as QString::number
    // prints them (%g). Returns false if a file cannot be opened; the directory must exist.
    bool exportLogs(const std::string &dir, const std::string &simulationType, const std::string &scenarioName) const
    {
        const std::string stem = dir + "/" + scenarioName + "_" + num(m_boxSize);
        FILE *f = std::fopen((stem + ".csv").c_str(), "a");
        FILE *d = std::fopen((stem + "_detail.csv").c_str(), "a");
        if (!f || !d) {
            if (f) std::fclose(f);
            if (d) std::fclose(d);
            return false;
        }
        std::string line = simulationType + ";";
        std::string rows[5];
        for (const auto &e : events) {
            line += num(e.together()) + ";";
            rows[0] += num(e.updateGrid) + ";";
            rows[1] += num(e.updateDensityPressure) + ";";
            rows[2] += num(e.updateForces) + ";";
            rows[3] += num(e.updateCollisions) + ";";
            rows[4] += num(e.integrate) + ";";
        }
        std::fputs((line + "\n").c_str(), f);
        static const char *labels[5] = {"Grid", "Density + pressure", "Forces", "Collisions", "Integrate"};
        std::string det = simulationType + "\n";
        for (int k = 0; k < 5; k++) det += std::string(labels[k]) + ";" + rows[k] + "\n";
        std::fputs((det + "\n\n").c_str(), d);
        std::fclose(f);
        std::fclose(d);
        return true;
    }

    // id-ordered state, as CGPUBaseParticleSimulator::integrate reads it back
    void readState(std::vector<float> &xyz, std::vector<float> &vel, std::vector<float> &rho)
    {
        xyz.resize(3 * m_particlesCount);
        vel.resize(3 * m_particlesCount);
        rho.resize(m_particlesCount);
        check(sph_download(m_ctx, xyz.data(), vel.data(), rho.data(), nullptr, nullptr));
    }

    // each pass returns its own milliseconds (0 when profiling is off): with profiling on, a
    // pass call waits for its work and its time is read right after it
    double passTime(int k)
    {
        if (!m_profiling) return 0.0;
        double ms[5];
        check(sph_pass_times(m_ctx, ms));
        return ms[k];
    }
    double updateGrid()
    {
        check(sph_pass_grid(m_ctx));
        return passTime(0);
    }
    double updateDensityPressure()
    {
        check(sph_pass_density(m_ctx));
        return passTime(1);
    }
    double updateForces()
    {
        check(sph_pass_forces(m_ctx));
        return passTime(2);
    }
    double updateCollisions() { return 0.0; }  // fused into updateForces
    double integrate() { return 0.0; }         // fused into updateForces

    // Front-end handoff without a synchronising readback: queue the id-ordered positions into
    // xyz (pinned host memory for an asynchronous copy; 3 floats per particle) and carry on
    // stepping; handoffWait() returns once they have landed.
    void handoffPositions(float *xyz) { check(sph_handoff_async(m_ctx, xyz, nullptr)); }
    void handoffWait() { check(sph_handoff_wait(m_ctx)); }

    // Re-time the force variants every `period` steps on real steps (0 = off); every variant
    // gives the same bits, so only the speed changes.
    void setOnlineTuning(int period) { check(sph_set_online_tuning(m_ctx, period)); }

private:
    static std::string num(double v)
    {
        char b[64];
        std::snprintf(b, sizeof b, "%g", v);
        return b;
    }

    void check(int rc, bool creating = false)
    {
        if (rc != SPH_OK) throw SphException(rc, sph_last_error(creating ? nullptr : m_ctx));
    }

    // FOUNTAIN emitter (src/CBaseParticleSimulator.cpp:187-210): 7 particles per step
    void generateParticles()
    {
        if (m_scenario != FOUNTAIN) return;
        const unsigned per = 7;
        if (m_particlesCount >= m_maxParticlesCount - per) return;
        const float hp = 0.0457f / 2.0f, q = 0.0457f / 4, oy = -m_boxSize / 2.0f;
        const float pts[21] = {0, oy, 0, -hp, oy, 0, hp, oy, 0, -q, oy, -hp, q, oy, -hp, -q, oy, hp, q, oy, hp};
        float vel[21];
        for (unsigned k = 0; k < per; k++) {
            vel[3 * k] = 0.0f;
            vel[3 * k + 1] = m_boxSize * 3.2f;
            vel[3 * k + 2] = 0.0f;
        }
        check(sph_append(m_ctx, 0, pts, vel, per));
        m_particlesCount += per;
    }

    float m_boxSize;
    SimulationScenario m_scenario;
    bool m_profiling;
    int m_precision;
    float m_gravity[3];
    sph_ctx *m_ctx = nullptr;
    unsigned long m_particlesCount = 0, m_maxParticlesCount = 0, m_totalIteration = 0;
    bool m_running = false;
    double m_last[5] = {0, 0, 0, 0, 0};
    unsigned long m_iterationSincePaused = 0;
    std::chrono::steady_clock::time_point m_t0 = std::chrono::steady_clock::now();
};

#endif  // CCUDAPARTICLESIMULATOR_HPP
