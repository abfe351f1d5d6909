// mps_io.cpp — JSON / .grid / .stl readers and .vtu / .pvd writers of the host driver.
#include "mps_io.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <sys/stat.h>
#include <sys/types.h>

namespace {

// ------------------------------------------------------------------ minimal JSON
// Objects, arrays, strings, numbers, booleans, null; // and /* */ comments are skipped
// (the reference parses with skip_comments, src/MpsInputOutput.cpp:126-129); with
// duplicate keys the last one wins.
struct JVal {
    enum Kind { NUL, BOOL, NUM, STR, ARR, OBJ } kind = NUL;
    bool b = false;
    double num = 0;
    std::string str;
    std::vector<JVal> arr;
    std::map<std::string, JVal> obj;
    const JVal* at(const char* k) const {
        if (kind != OBJ) return nullptr;
        auto it = obj.find(k);
        return it == obj.end() ? nullptr : &it->second;
    }
};

struct JParser {
    const std::string& s;
    size_t p = 0;
    std::string err;
    explicit JParser(const std::string& t) : s(t) {}
    void ws() {
        while (p < s.size()) {
            char c = s[p];
            if (c == ' ' || c == '\t' || c == '\n' || c == '\r') { p++; continue; }
            if (c == '/' && p + 1 < s.size() && s[p + 1] == '/') { while (p < s.size() && s[p] != '\n') p++; continue; }
            if (c == '/' && p + 1 < s.size() && s[p + 1] == '*') {
                size_t e = s.find("*/", p + 2);
                p = (e == std::string::npos) ? s.size() : e + 2;
                continue;
            }
            break;
        }
    }
    bool fail(const char* m) { if (err.empty()) { err = m; err += " at byte " + std::to_string(p); } return false; }
    bool str(std::string& out) {
        if (s[p] != '"') return fail("expected string");
        p++;
        out.clear();
        while (p < s.size() && s[p] != '"') {
            if (s[p] == '\\' && p + 1 < s.size()) {
                char e = s[p + 1];
                out += (e == 'n') ? '\n' : (e == 't') ? '\t' : e;
                p += 2;
            } else out += s[p++];
        }
        if (p >= s.size()) return fail("unterminated string");
        p++;
        return true;
    }
    bool val(JVal& v) {
        ws();
        if (p >= s.size()) return fail("unexpected end");
        char c = s[p];
        if (c == '{') {
            v.kind = JVal::OBJ;
            p++;
            ws();
            if (s[p] == '}') { p++; return true; }
            while (true) {
                ws();
                std::string k;
                if (!str(k)) return false;
                ws();
                if (s[p] != ':') return fail("expected ':'");
                p++;
                JVal x;
                if (!val(x)) return false;
                v.obj[k] = std::move(x);
                ws();
                if (s[p] == ',') { p++; continue; }
                if (s[p] == '}') { p++; return true; }
                return fail("expected ',' or '}'");
            }
        }
        if (c == '[') {
            v.kind = JVal::ARR;
            p++;
            ws();
            if (s[p] == ']') { p++; return true; }
            while (true) {
                JVal x;
                if (!val(x)) return false;
                v.arr.push_back(std::move(x));
                ws();
                if (s[p] == ',') { p++; continue; }
                if (s[p] == ']') { p++; return true; }
                return fail("expected ',' or ']'");
            }
        }
        if (c == '"') { v.kind = JVal::STR; return str(v.str); }
        if (!s.compare(p, 4, "true")) { v.kind = JVal::BOOL; v.b = true; p += 4; return true; }
        if (!s.compare(p, 5, "false")) { v.kind = JVal::BOOL; v.b = false; p += 5; return true; }
        if (!s.compare(p, 4, "null")) { v.kind = JVal::NUL; p += 4; return true; }
        char* end = nullptr;
        v.num = std::strtod(s.c_str() + p, &end);
        if (end == s.c_str() + p) return fail("bad value");
        v.kind = JVal::NUM;
        p = end - s.c_str();
        return true;
    }
};

// json::value(key, default) of nlohmann, for the kinds used here
double num(const JVal* o, const char* k, double d) {
    const JVal* v = o ? o->at(k) : nullptr;
    if (!v) return d;
    if (v->kind == JVal::NUM) return v->num;
    if (v->kind == JVal::BOOL) return v->b ? 1.0 : 0.0;
    return d;
}
bool flag(const JVal* o, const char* k, bool d) {
    const JVal* v = o ? o->at(k) : nullptr;
    if (!v) return d;
    if (v->kind == JVal::BOOL) return v->b;
    if (v->kind == JVal::NUM) return v->num != 0;
    return d;
}
std::string text(const JVal* o, const char* k, const char* d) {
    const JVal* v = o ? o->at(k) : nullptr;
    return (v && v->kind == JVal::STR) ? v->str : std::string(d);
}
// je.at(section): a missing section is reported and its keys keep their defaults
const JVal* section(const JVal* o, const char* k) {
    const JVal* v = o ? o->at(k) : nullptr;
    if (!v) std::printf("[json.exception.out_of_range.403] key '%s' not found\n", k);
    return v;
}

}  // namespace

int readInputFile(const std::string& jsonPath, CaseInput& c, std::string& err) {
    std::ifstream f(jsonPath);
    if (!f) { err = "cannot open " + jsonPath; return MPSGPU_ERR_ARG; }
    std::stringstream ss;
    ss << f.rdbuf();
    std::string txt = ss.str();
    JParser jp(txt);
    JVal root;
    if (!jp.val(root) || root.kind != JVal::OBJ) { err = "JSON INPUT FILE ERROR: " + jp.err; return MPSGPU_ERR_ARG; }
    MpsParams& P = c.params;
    std::memset(&P, 0, sizeof(P));
    const JVal* fl = section(&root, "flags");
    P.wallType = (int)num(fl, "wall_type", 1);
    P.femOn = flag(fl, "fem_MESH", false);
    P.forcedOn = flag(fl, "forced_MESH", false);
    const JVal* vtu = fl ? section(fl, "output_VTU") : nullptr;
    c.out.vtuType = (int)num(vtu, "type", 0);
    c.out.freeSurfWall = flag(vtu, "only_freeSurface", false);   // key as read by the reference
    c.out.pnd = flag(vtu, "pnd", false);
    c.out.neigh = flag(vtu, "neigh", false);
    c.out.deviation = flag(vtu, "deviation", false);
    c.out.concentration = flag(vtu, "concentration", false);
    c.out.auxiliar = flag(vtu, "auxiliar", false);
    c.out.nonNewtonian = flag(vtu, "non_newtonian", false);
    const JVal* pn = section(&root, "pathNames");
    c.gridFile = text(pn, "particle_grid_file", "oops");
    c.meshRigidFile = text(pn, "mesh_rigid_file", "oops");
    c.vtuFolder = text(pn, "vtu_output_folder", "oops");
    const JVal* dom = section(&root, "domain");
    const JVal* dmin = dom ? section(dom, "min") : nullptr;
    const JVal* dmax = dom ? section(dom, "max") : nullptr;
    const char* xyz[3] = {"x", "y", "z"};
    for (int k = 0; k < 3; k++) { P.domainMin[k] = num(dmin, xyz[k], 0.0); P.domainMax[k] = num(dmax, xyz[k], 0.0); }
    const JVal* bnd = dom ? section(dom, "boundary") : nullptr;
    P.domainTypeBC = (int)num(bnd, "type", 0);
    P.limitTypeBC = (int)num(bnd, "limit", 0);
    const JVal* ph = section(&root, "physical");
    P.densityFluid = num(ph, "fluid_density", 1000.0);
    P.densityWall = num(ph, "wall_density", 1000.0);
    P.KNM_VS1 = num(ph, "kinematic_visc", 0.000001);
    P.fluidType = (int)num(ph, "fluid_type", 0);
    const JVal* gr = ph ? section(ph, "gravity") : nullptr;
    P.gravity[0] = num(gr, "x", 0.0); P.gravity[1] = num(gr, "y", 0.0); P.gravity[2] = num(gr, "z", -9.81);
    const JVal* rh = ph ? section(ph, "rheological") : nullptr;
    P.KNM_VS2 = num(rh, "kinematic_visc_phase_2", 0.000001);
    P.DNS_FL1 = num(rh, "fluid_density_phase_1", 1000.0);
    P.DNS_FL2 = num(rh, "fluid_density_phase_2", 1540.0);
    const JVal* nu = section(&root, "numerical");
    P.dim = num(nu, "dimension", 3.0);
    P.partDist = num(nu, "particle_dist", 0.01);
    P.timeStep = num(nu, "time_step", 0.0005);
    P.timeSimulation = num(nu, "final_time", 1.0);
    P.iterOutput = (int)num(nu, "iter_output", 80);
    P.cflNumber = num(nu, "CFL_number", 0.2);
    P.weightType = (int)num(nu, "weight_type", 0);
    P.slipCondition = (int)num(nu, "slip_condition", 0);
    const JVal* re = nu ? section(nu, "effective_radius") : nullptr;
    P.reS = num(re, "small", 2.1);
    P.reL = num(re, "large", 2.1);
    const JVal* gd = nu ? section(nu, "gradient") : nullptr;
    P.gradientType = (int)num(gd, "type", 0);
    P.gradientCorrection = flag(gd, "correction", false);
    P.relaxPress = num(gd, "relax_fact", 1.0);
    P.mpsType = (int)num(nu, "mps_type", 1);
    const JVal* ex = nu ? section(nu, "explicit_mps") : nullptr;
    const JVal* eq = ex ? section(ex, "equation_state") : nullptr;
    P.soundSpeed = num(eq, "speed_sound", 15.0);
    P.gamma = num(eq, "gamma", 7.0);
    const JVal* im = nu ? section(nu, "semi_implicit_mps") : nullptr;
    P.solverType = (int)num(im, "solver_type", 0);
    const JVal* wk = im ? section(im, "weak_compressibility") : nullptr;
    P.alphaCompressibility = num(wk, "alpha", 0.000001);
    const JVal* srcs = im ? section(im, "source_term") : nullptr;
    P.relaxPND = num(srcs, "relax_pnd", 0.001);
    const JVal* sh = nu ? section(nu, "particle_shifting") : nullptr;
    P.shiftingType = (int)num(sh, "type", 2);
    P.dri = num(sh, "DRI", 0.01);
    P.coefA = num(sh, "coef_A", 2.0);
    P.machNumber = num(sh, "mach_number", 0.1);
    const JVal* pd = nu ? section(nu, "pnd") : nullptr;
    P.pndType = (int)num(pd, "type", 0);
    P.diffusiveCoef = num(pd, "diffusive_coeff", 0.35);
    const JVal* wf = nu ? section(nu, "wall_repulsive_force") : nullptr;
    P.repulsiveForceType = (int)num(wf, "type", 2);
    P.reRepulsiveForce = num(wf, "re", 0.5);
    P.expectMaxVelocity = num(wf, "maxVel", 6.0);
    const JVal* wc = wf ? section(wf, "coefficient") : nullptr;
    P.repForceCoefMitsume = num(wc, "Mitsume", 40000000.0);
    P.repForceCoefLennardJones = num(wc, "Lennard-Jones", 2.0);
    P.repForceCoefMonaghanKajtar = num(wc, "Monaghan-Kajtar", 1.0);
    P.EPS_RE = num(wf, "eps_re", 0.01);
    const JVal* fs = nu ? section(nu, "free_surface_threshold") : nullptr;
    P.freeSurfType = (int)num(fs, "type", 0);
    P.pndThreshold = num(fs, "pnd", 0.98);
    P.neighThreshold = num(fs, "neigh", 0.85);
    P.npcdThreshold = num(fs, "NPCD", 0.20);
    P.thetaThreshold = num(fs, "ARC", 45.0);
    P.normThreshold = num(fs, "normal", 0.1);
    const JVal* co = nu ? section(nu, "particle_collision") : nullptr;
    P.collisionType = (int)num(co, "type", 0);
    P.collisionRatio = num(co, "ratio", 0.20);
    P.distLimitRatio = num(co, "dist_limit_ratio", 0.85);
    P.lambdaCollision = num(co, "lambda", 0.20);
    const JVal* pt = nu ? section(nu, "particle_type") : nullptr;
    P.ghost = (int)num(pt, "ghost", -1);
    P.fluid = (int)num(pt, "fluid", 0);
    P.wall = (int)num(pt, "wall", 2);
    P.dummyWall = (int)num(pt, "dummyWall", 3);
    const JVal* bt = nu ? section(nu, "boundary_type") : nullptr;
    P.surface = (int)num(bt, "free_surface", 1);
    P.inner = (int)num(bt, "inner", 0);
    P.other = (int)num(bt, "other", -1);
    // optional GPU section
    if (const JVal* g = root.at("gpu")) {
        std::string s = text(g, "solver", "plain");
        c.gpu.solver = (s == "mixed") ? MPSGPU_SOLVER_MIXED : MPSGPU_SOLVER_PLAIN_FP64;
        std::string w = text(g, "warm_start", "previous");
        c.gpu.warmStart = (w == "mlp")            ? MPSGPU_WARM_MLP
                          : (w == "zero")         ? MPSGPU_WARM_ZERO
                          : (w == "extrapolate")  ? MPSGPU_WARM_EXTRAPOLATE
                          : (w == "extrapolate2") ? MPSGPU_WARM_EXTRAPOLATE2
                                                  : MPSGPU_WARM_PREVIOUS;
        const JVal* t = g->at("tol");
        if (t && t->kind == JVal::STR && t->str == "eigen")
            c.gpu.tol = 2.220446049250313e-16;   // Eigen's default: the machine epsilon
        else
            c.gpu.tol = num(g, "tol", 1e-8);
        c.gpu.maxIter = (int)num(g, "max_iter", 0);
        c.gpu.mlpWeights = text(g, "mlp_weights", "");
    }
    // checks of src/MpsInputOutput.cpp:531-544
    if (P.partDist * P.partDist <= 10.0 * 2.220446049250313e-16) {
        err = "operations using squared particle distance lower than the machine double precision";
        return MPSGPU_ERR_ARG;
    }
    if ((P.mpsType == 2 || P.mpsType == 3) && (P.pndType == 1 || P.pndType == 2)) {
        err = "set 'pnd-type to 0' in the json file for incompressible MPS";
        return MPSGPU_ERR_ARG;
    }
    int e = readGridFile(c.gridFile, c, err);
    if (e) return e;
    if (P.wallType == 1) {
        e = readStlFile(c.meshRigidFile, c.tri, err);
        if (e) return e;
    }
    return 0;
}

// .grid: "0", N, then "type x y z vx vy vz p p_av" per particle (src/MpsInputOutput.cpp:659-776)
int readGridFile(const std::string& path, CaseInput& c, std::string& err) {
    FILE* fp = std::fopen(path.c_str(), "r");
    if (!fp) { err = "Error opening grid file " + path; return MPSGPU_ERR_ARG; }
    int zero = 0, n = 0;
    if (std::fscanf(fp, "%d", &zero) != 1 || std::fscanf(fp, "%d", &n) != 1 || n <= 0) {
        std::fclose(fp);
        err = "bad grid header in " + path;
        return MPSGPU_ERR_ARG;
    }
    c.type.resize(n); c.pos.resize(3 * (size_t)n); c.vel.resize(3 * (size_t)n); c.press.resize(n);
    for (int i = 0; i < n; i++) {
        int t;
        double b[8];
        if (std::fscanf(fp, "%d %lf %lf %lf %lf %lf %lf %lf %lf", &t, &b[0], &b[1], &b[2], &b[3], &b[4], &b[5], &b[6], &b[7]) != 9) {
            std::fclose(fp);
            err = "truncated grid file " + path;
            return MPSGPU_ERR_ARG;
        }
        c.type[i] = t;
        for (int k = 0; k < 3; k++) { c.pos[3 * i + k] = b[k]; c.vel[3 * i + k] = b[3 + k]; }
        c.press[i] = b[6];
    }
    std::fclose(fp);
    return 0;
}

int readStlFile(const std::string& path, std::vector<double>& tri, std::string& err) {
    std::ifstream f(path, std::ios::binary);
    if (!f) { err = "IOError: " + path + " could not be opened"; return MPSGPU_ERR_ARG; }
    std::string data((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    tri.clear();
    if (data.size() >= 84) {
        uint32_t nt = 0;
        std::memcpy(&nt, data.data() + 80, 4);
        if (data.size() == 84 + 50ull * nt) {   // binary
            for (uint32_t t = 0; t < nt; t++) {
                const char* r = data.data() + 84 + 50ull * t + 12;
                for (int k = 0; k < 9; k++) {
                    float v;
                    std::memcpy(&v, r + 4 * k, 4);
                    tri.push_back(v);
                }
            }
            return 0;
        }
    }
    std::istringstream in(data);   // ASCII: "vertex x y z" triples
    std::string w;
    while (in >> w) {
        if (w == "vertex") {
            double x, y, z;
            in >> x >> y >> z;
            tri.push_back(x); tri.push_back(y); tri.push_back(z);
        }
    }
    if (tri.empty() || tri.size() % 9) { err = "IOError: STL mesh " + path + " could not be read"; return MPSGPU_ERR_ARG; }
    return 0;
}

// MpsInputOutput::writeVtuAscii, src/MpsInputOutput.cpp:1313-1580 (same arrays and names)
int writeVtuAscii(const std::string& folder, int fileNumber, const OutputFlags& fl, const VtuFields& v, bool polygon) {
    char name[1024];
    std::snprintf(name, sizeof(name), "%s/output%05d.vtu", folder.c_str(), fileNumber);
    FILE* fp = std::fopen(name, "w");
    if (!fp) return MPSGPU_ERR_ARG;
    int n = v.n;
    std::fprintf(fp, "<?xml version='1.0' encoding='UTF-8'?>\n");
    std::fprintf(fp, "<VTKFile xmlns='VTK' byte_order='LittleEndian' version='0.1' type='UnstructuredGrid'>\n");
    std::fprintf(fp, "  <UnstructuredGrid>\n");
    std::fprintf(fp, "    <Piece NumberOfCells='%d' NumberOfPoints='%d'>\n", n, n);
    std::fprintf(fp, "      <Points>\n");
    std::fprintf(fp, "        <DataArray type='Float32' Name='Position' NumberOfComponents='3' format='ascii'>\n          ");
    for (int i = 0; i < n; i++) std::fprintf(fp, "%lf %lf %lf ", v.pos[3 * i], v.pos[3 * i + 1], v.pos[3 * i + 2]);
    std::fprintf(fp, "\n        </DataArray>\n");
    std::fprintf(fp, "      </Points>\n");
    std::fprintf(fp, "      <PointData>\n");
    auto vec = [&](const char* nm, const std::vector<double>& a) {
        std::fprintf(fp, "        <DataArray type='Float32' Name='%s' NumberOfComponents='3' format='ascii'>\n", nm);
        for (int i = 0; i < n; i++) std::fprintf(fp, "%f %f %f ", (float)a[3 * i], (float)a[3 * i + 1], (float)a[3 * i + 2]);
        std::fprintf(fp, "\n        </DataArray>\n");
    };
    auto sca = [&](const char* nm, const std::vector<double>& a) {
        std::fprintf(fp, "        <DataArray type='Float32' Name='%s' format='ascii'>\n", nm);
        for (int i = 0; i < n; i++) std::fprintf(fp, "%f ", (float)a[i]);
        std::fprintf(fp, "\n        </DataArray>\n");
    };
    auto ints = [&](const char* nm, const std::vector<int>& a) {
        std::fprintf(fp, "        <DataArray type='Int32' Name='%s' format='ascii'>\n", nm);
        for (int i = 0; i < n; i++) std::fprintf(fp, "%d ", a[i]);
        std::fprintf(fp, "\n        </DataArray>\n");
    };
    vec("Velocity", v.vel);
    sca("pressure", v.press);
    ints("BC", v.bc);
    if (fl.pnd) { sca("pnd", v.pndi); sca("pndSmall", v.pndSmall); }
    if (fl.neigh) ints("nNeigh", v.numNeigh);
    if (fl.deviation) { vec("npcdDeviation", v.npcd); vec("polygonNormal", v.polyNormal); }
    if (fl.concentration) { sca("concentration", v.conc); vec("GradCi", v.gradC); }
    if (fl.auxiliar) {
        ints("ParticleType", v.type);
        if (polygon) ints("nearMeshType", std::vector<int>(n, 0));
    }
    std::fprintf(fp, "      </PointData>\n");
    std::fprintf(fp, "      <Cells>\n");
    std::fprintf(fp, "        <DataArray type='Int32' Name='connectivity' format='ascii'>\n");
    for (int i = 0; i < n; i++) std::fprintf(fp, "%d ", i);
    std::fprintf(fp, "\n        </DataArray>\n");
    std::fprintf(fp, "        <DataArray type='Int32' Name='offsets' format='ascii'>\n");
    for (int i = 0; i < n; i++) std::fprintf(fp, "%d ", i + 1);
    std::fprintf(fp, "\n        </DataArray>\n");
    std::fprintf(fp, "        <DataArray type='UInt8' Name='types' format='ascii'>\n");
    for (int i = 0; i < n; i++) std::fprintf(fp, "1 ");
    std::fprintf(fp, "\n        </DataArray>\n");
    std::fprintf(fp, "      </Cells>\n");
    std::fprintf(fp, "    </Piece>\n");
    std::fprintf(fp, "  </UnstructuredGrid>\n");
    std::fprintf(fp, "</VTKFile>\n");
    std::fclose(fp);
    return 0;
}

// MpsInputOutput::writePvd, src/MpsInputOutput.cpp:1878-1933 (creates the output folder)
int writePvd(const std::string& folder, double timeSimulation, double dt, int iterOutput) {
    std::string base = folder;
    size_t found = base.find('/');
    if (found != std::string::npos) base.erase(0, found + 1);
    if (mkdir(folder.c_str(), 0777) == -1) std::printf("Unable to create OUTPUT directory or it has already been created!\n");
    else std::printf("Directory created.\n");
    std::string pvd = folder + ".pvd";
    FILE* fp = std::fopen(pvd.c_str(), "w");
    if (!fp) return MPSGPU_ERR_ARG;
    int nIter = (int)std::ceil(timeSimulation / dt);
    std::fprintf(fp, "<VTKFile type='Collection' version='0.1' byte_order='LittleEndian'>\n");
    std::fprintf(fp, "  <Collection>\n");
    int j = 0;
    for (int i = 0; i < nIter; i++)
        if (i % iterOutput == 0) {
            std::fprintf(fp, "    <DataSet timestep='%.6f' group='A' part='0' file='%s/output%05d.vtu'/>\n", dt * i,
                         base.c_str(), j);
            j++;
        }
    std::fprintf(fp, "  </Collection>\n");
    std::fprintf(fp, "</VTKFile>\n");
    std::fclose(fp);
    return 0;
}
