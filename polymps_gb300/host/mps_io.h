// mps_io.h — host-side formats of the PolyMPS drop-in: JSON input (the schema and
// defaults of MpsInputOutput::readInputFile, src/MpsInputOutput.cpp:58-641), the .grid
// particle file (src/MpsInputOutput.cpp:645-857), STL meshes (binary or ASCII, what
// igl::readSTL accepts), and the ASCII .vtu/.pvd writers
// (src/MpsInputOutput.cpp:1313-1580, :1878-1933).
#pragma once
#include <string>
#include <vector>
#include "mpsgpu.h"

struct OutputFlags {
    int vtuType = 0;
    bool freeSurfWall = false, pnd = false, neigh = false, deviation = false, concentration = false;
    bool auxiliar = false, nonNewtonian = false;
};

struct GpuOptions {               // optional "gpu" section (new knobs, no reference counterpart)
    int solver = MPSGPU_SOLVER_PLAIN_FP64;
    int warmStart = MPSGPU_WARM_PREVIOUS;
    // PPE relative tolerance: 1e-8 unless the JSON says otherwise; "eigen" selects Eigen's
    // default, the machine epsilon, which the reference runs with (it never calls
    // setTolerance: src/MpsPressure.cpp:427 is commented out)
    double tol = 1e-8;
    int maxIter = 0;
    std::string mlpWeights;       // .bin: MPSGPU_MLP_NPARAM + 32 floats
};

struct CaseInput {
    MpsParams params{};
    OutputFlags out;
    GpuOptions gpu;
    std::string gridFile, meshRigidFile, vtuFolder;
    std::vector<int> type;
    std::vector<double> pos, vel, press;
    std::vector<double> tri;      // ntri * 9
};

// Reads the JSON file and the .grid / .stl it names.  Returns 0 or an MPSGPU_ERR_* code;
// err receives a message.
int readInputFile(const std::string& jsonPath, CaseInput& c, std::string& err);
int readGridFile(const std::string& path, CaseInput& c, std::string& err);
int readStlFile(const std::string& path, std::vector<double>& tri, std::string& err);

struct VtuFields {
    int n = 0;
    std::vector<double> pos, vel, press, pndi, pndSmall, npcd, polyNormal, conc, gradC;
    std::vector<int> bc, numNeigh, type;
};
int writeVtuAscii(const std::string& folder, int fileNumber, const OutputFlags& f, const VtuFields& v,
                  bool polygon);
int writePvd(const std::string& folder, double timeSimulation, double dt, int iterOutput);
