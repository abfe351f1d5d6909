// mps_driver.cpp — command-line driver of the GB300 PolyMPS path, the counterpart of
// main() and mainLoopOfSimulation (src/main.cpp:75-469): reads the reference's JSON,
// .grid and .stl inputs, runs the step loop on the GPU through the C ABI, prints the
// progress line of displayInfo every 100 iterations and writes .vtu/.pvd output every
// iter_output iterations.
//
//   mps_gb300 <input.json> [--max-steps N] [--no-output] [--check-input params.bin]
// --check-input parses the JSON, .grid and .stl, derives the constants and checks the
// switches on the host only (no GPU), writes the MpsParams as read (before derivation)
// as raw bytes to the given file, prints one status line and exits with the status code.
// Without an argument the input name is read from stdin relative to input/ with .json
// appended, as the reference does (src/MpsInputOutput.cpp:89-109).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include "mps_io.h"

static double now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

#define TRY(call)                                                                             \
    do {                                                                                      \
        int _e = (call);                                                                      \
        if (_e) {                                                                             \
            std::fprintf(stderr, "%s failed (%d): %s\n", #call, _e, mpsgpu_last_error(h));   \
            return 2;                                                                         \
        }                                                                                     \
    } while (0)

int main(int argc, char** argv) {
    std::printf("Start PolyMPS (GB300).\n");
    std::string json;
    long long maxSteps = -1;
    bool output = true;
    std::string checkPath;
    for (int a = 1; a < argc; a++) {
        if (!std::strcmp(argv[a], "--max-steps") && a + 1 < argc) maxSteps = std::atoll(argv[++a]);
        else if (!std::strcmp(argv[a], "--no-output")) output = false;
        else if (!std::strcmp(argv[a], "--check-input") && a + 1 < argc) checkPath = argv[++a];
        else json = argv[a];
    }
    if (json.empty()) {
        char name[1000];
        std::printf("Enter the name of the MPS input file:\n");
        if (std::scanf("%999s", name) != 1) return 1;
        json = std::string("input/") + name + ".json";
    }
    CaseInput c;
    std::string err;
    double t0 = now();
    int rc = readInputFile(json, c, err);
    int n = (int)c.type.size();
    if (!checkPath.empty()) {
        // the parameters as read (before derivation scales the radii and sets the domain)
        if (FILE* f = std::fopen(checkPath.c_str(), "wb")) {
            std::fwrite(&c.params, sizeof(MpsParams), 1, f);
            std::fclose(f);
        }
        MpsParams d = c.params;
        if (!rc && (rc = mpsgpu_params_derive(&d, n, c.pos.data())) != 0) err = mpsgpu_last_error(nullptr);
        if (!rc && (rc = mpsgpu_check_params(&d)) != 0) err = mpsgpu_last_error(nullptr);
        std::printf("check-input status %d particles %d triangles %d: %s\n", rc, n, (int)(c.tri.size() / 9),
                    rc ? err.c_str() : "ok");
        return rc;
    }
    if (rc) {
        std::fprintf(stderr, "%s\n", err.c_str());
        return rc;
    }
    mpsgpu_t h = nullptr;
    TRY(mpsgpu_params_derive(&c.params, n, c.pos.data()));
    MpsMesh mesh{(int)(c.tri.size() / 9), c.tri.data()};
    TRY(mpsgpu_create(&c.params, n, c.type.data(), c.pos.data(), c.vel.data(), c.press.data(),
                      c.params.wallType == 1 ? &mesh : nullptr, &h));
    if (c.gpu.warmStart == MPSGPU_WARM_MLP) {
        std::vector<float> w(MPSGPU_MLP_NPARAM + 2 * MPSGPU_MLP_NFEAT);
        FILE* f = std::fopen(c.gpu.mlpWeights.c_str(), "rb");
        if (!f || std::fread(w.data(), sizeof(float), w.size(), f) != w.size()) {
            std::fprintf(stderr, "cannot read MLP weights %s\n", c.gpu.mlpWeights.c_str());
            return 1;
        }
        std::fclose(f);
        TRY(mpsgpu_mlp_set_weights(h, w.data(), w.data() + MPSGPU_MLP_NPARAM));
    }
    TRY(mpsgpu_set_solver(h, c.gpu.solver, c.gpu.warmStart, c.gpu.tol, c.gpu.maxIter));
    std::printf("Initial Step... ");
    TRY(mpsgpu_initialize(h));
    if (output) writePvd(c.vtuFolder, c.params.timeSimulation, c.params.timeStep, c.params.iterOutput);
    std::printf("OK\n\nStart Main Loop of Simulation\n\n");
    const MpsParams& P = c.params;
    int iter = 0, fileNumber = 0;
    double time = 0.0;
    MpsStepStats st{};
    st.numParticles = n;
    VtuFields v;
    while (true) {
        if (iter % 100 == 0) {
            int sec = (int)(now() - t0);
            std::printf("Iteration: %5dth Time: %lfsec Num. Particles: %d Max Velocity: %lfm/s Courant: %lf", iter, time,
                        st.numParticles, st.velMax, st.CFLcurrent);
            if (P.mpsType == 2 || P.mpsType == 3) std::printf(" Solver iterations: %3d Estimated error: %.2e", st.ppeIterations, st.ppeRelResidual);
            std::printf(" RunTime: %02dh%02dm%02dsec\n", sec / 3600, (sec / 60) % 60, sec % 60);
        }
        if (output && iter % P.iterOutput == 0 && c.out.vtuType == 1) {
            // binary: formatted from the device buffers by the library
            char name[1024];
            std::snprintf(name, sizeof(name), "%s/output%05d.vtu", c.vtuFolder.c_str(), fileNumber);
            unsigned int groups = (c.out.pnd ? MPSGPU_VTU_PND : 0u) | (c.out.neigh ? MPSGPU_VTU_NEIGH : 0u) |
                                  (c.out.deviation ? MPSGPU_VTU_DEVIATION : 0u) |
                                  (c.out.concentration ? MPSGPU_VTU_CONCENTRATION : 0u) |
                                  (c.out.auxiliar ? MPSGPU_VTU_AUXILIAR : 0u);
            TRY(mpsgpu_write_vtu(h, name, groups));
            fileNumber++;
        } else if (output && iter % P.iterOutput == 0) {
            int cur = 0;
            TRY(mpsgpu_num_particles(h, &cur));
            v.n = cur;
            v.pos.resize(3 * cur); v.vel.resize(3 * cur); v.press.resize(cur); v.bc.resize(cur);
            v.pndi.resize(cur); v.pndSmall.resize(cur); v.numNeigh.resize(cur); v.npcd.resize(3 * cur);
            v.polyNormal.resize(3 * cur); v.conc.resize(cur); v.gradC.resize(3 * cur); v.type.resize(cur);
            TRY(mpsgpu_get_field(h, MPS_F_POS, v.pos.data()));
            TRY(mpsgpu_get_field(h, MPS_F_VEL, v.vel.data()));
            TRY(mpsgpu_get_field(h, MPS_F_PRESS, v.press.data()));
            TRY(mpsgpu_get_field(h, MPS_F_BC, v.bc.data()));
            if (c.out.pnd) { TRY(mpsgpu_get_field(h, MPS_F_PNDI, v.pndi.data())); TRY(mpsgpu_get_field(h, MPS_F_PNDSMALL, v.pndSmall.data())); }
            if (c.out.neigh) TRY(mpsgpu_get_field(h, MPS_F_NUMNEIGH, v.numNeigh.data()));
            if (c.out.deviation) { TRY(mpsgpu_get_field(h, MPS_F_NPCD, v.npcd.data())); TRY(mpsgpu_get_field(h, MPS_F_POLYNORMAL, v.polyNormal.data())); }
            if (c.out.concentration) { TRY(mpsgpu_get_field(h, MPS_F_CONC, v.conc.data())); TRY(mpsgpu_get_field(h, MPS_F_GRADC, v.gradC.data())); }
            if (c.out.auxiliar) TRY(mpsgpu_get_field(h, MPS_F_TYPE, v.type.data()));
            writeVtuAscii(c.vtuFolder, fileNumber, c.out, v, P.wallType == 1);
            fileNumber++;
        }
        TRY(mpsgpu_step(h, &st));
        iter++;
        time += P.timeStep;
        if (time > P.timeSimulation) break;
        if (maxSteps >= 0 && iter >= maxSteps) break;
    }
    std::printf("Steps: %d  N: %d  last PPE iterations %d relres %.2e  wall %.2f s\n", iter, st.numParticles,
                st.ppeIterations, st.ppeRelResidual, now() - t0);
    mpsgpu_destroy(h);
    std::printf("End PolyMPS.\n");
    return 0;
}
