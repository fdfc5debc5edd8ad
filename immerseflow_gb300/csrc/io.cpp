// io.cpp -- the reference's file surface: inputs.txt, grid files, Tecplot.
//
// inputs.txt uses the reference grammar (src/main.cu:10-59): a line that
// contains a keyword announces that the NEXT line holds its values; lines
// starting with '=' or '_' and empty lines are skipped.  The reference
// keywords are matched first and in the same order.  Extension keywords
// (solver mode, precision, boundary types, body, tolerances, ...) contain
// none of the reference's keyword substrings, so the reference parser
// ignores them and reads an extended file exactly as before.
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>

#include "ifx_host.h"

namespace ifx {

thread_local std::string g_last_error;

ifx_status set_error(ifx_status st, const std::string& msg) {
    g_last_error = msg;
    return st;
}

}  // namespace ifx

using ifx::set_error;

extern "C" const char* ifx_last_error(void) { return ifx::g_last_error.c_str(); }

extern "C" const char* ifx_status_string(ifx_status s) {
    switch (s) {
        case IFX_OK: return "ok";
        case IFX_ERR_ARG: return "invalid argument";
        case IFX_ERR_IO: return "file i/o error";
        case IFX_ERR_PARSE: return "parse error";
        case IFX_ERR_CUDA: return "CUDA error";
        case IFX_ERR_NOMEM: return "out of memory";
        case IFX_ERR_NOT_CONVERGED: return "iteration cap reached";
        case IFX_ERR_DIVERGED: return "non-finite state";
        case IFX_ERR_BUDGET: return "HBM budget exceeded";
        case IFX_ERR_STATE: return "invalid state";
        case IFX_ERR_NODEVICE: return "no CUDA device";
        case IFX_ERR_GEOMETRY: return "moving body left the domain or outgrew its ghost slots";
    }
    return "unknown status";
}

extern "C" const char* ifx_version(void) { return "immerseflow_gb300 0.1 (sm_103a)"; }

extern "C" void ifx_config_default(ifx_config* c) {
    std::memset(c, 0, sizeof(*c));
    // inputs/inputs.txt of the reference
    c->restart = 0;
    c->restart_time = 9;
    c->nx = 50;
    c->ny = 50;
    c->lx = 10.0;
    c->ly = 5.0;
    c->w_ad = 1;
    c->w_ppe = 1;
    c->ad_itermax = 25;
    c->ppe_itermax = 100000;
    c->ad_solver = 1;
    c->ppe_solver = 1;
    c->error_max = 1e-6;
    c->tmax = 100.0;
    c->dt = 0.001;
    c->re = 150.0;
    c->mu = 0.01;
    c->write_interval = 1000;
    c->mode = IFX_MODE_REFERENCE;
    c->precision = IFX_PREC_FP64;
    c->init = IFX_INIT_VORTEX;
    for (int s = 0; s < 4; s++) {
        c->bc_type[s] = IFX_BC_WALL;
        c->bc_u[s] = 1.0;  // the reference's all-wall u = 1, v = 0 ghost rule
        c->bc_v[s] = 0.0;
    }
    c->outflow_uc = 1.0;
    c->body = IFX_BODY_NONE;
    c->body_a = c->body_b = 0.5;
    c->ppe_tol = 1e-8;
    c->ad_tol = 1e-12;
    c->mg_pre = 2;
    c->mg_post = 2;
    c->mg_omega = 0.8;
    c->mixed_inner = 8;
    c->coarse_sweeps = 40;
    c->restart_drop = 1e-4;
    c->restart_every = 25;
    c->force_ref_u = 1.0;
    c->force_ref_len = 1.0;
    c->ppe_method = IFX_PPE_JACOBI;
    c->relax_ad = 1.0;
    c->relax_ppe = 1.0;
    std::snprintf(c->xgrid, IFX_PATH_MAX, "xgrid.dat2");
    std::snprintf(c->ygrid, IFX_PATH_MAX, "ygrid.dat2");
}

namespace {

std::string dir_of(const std::string& p) {
    size_t k = p.find_last_of('/');
    return k == std::string::npos ? std::string(".") : p.substr(0, k);
}

bool parse_bc(const std::string& w, int* out) {
    if (w == "wall") *out = IFX_BC_WALL;
    else if (w == "inflow") *out = IFX_BC_INFLOW;
    else if (w == "outflow") *out = IFX_BC_OUTFLOW;
    else if (w == "slip") *out = IFX_BC_SLIP;
    else return false;
    return true;
}

}  // namespace

extern "C" ifx_status ifx_config_read(const char* path, ifx_config* c) {
    if (!path || !c) return set_error(IFX_ERR_ARG, "ifx_config_read: null argument");
    std::ifstream f(path);
    if (!f.is_open()) return set_error(IFX_ERR_IO, std::string("Unable to open file: ") + path);
    ifx_config_default(c);
    std::string xg = "xgrid.dat2", yg = "ygrid.dat2";
    std::string line;
    int nlines = 0;
    auto bad = [&](const char* what) {
        return set_error(IFX_ERR_PARSE, std::string(path) + ": bad values after '" + what + "'");
    };
    while (std::getline(f, line)) {
        if (line.empty() || line[0] == '=' || line[0] == '_') continue;
        std::istringstream iss;
        auto next = [&]() -> bool {
            if (!std::getline(f, line)) return false;
            iss.str(line);
            iss.clear();
            return true;
        };
        // reference keywords, same order as src/main.cu:27-51
        if (line.find("Restart") != std::string::npos) {
            if (!next() || !(iss >> c->restart >> c->restart_time)) return bad("Restart");
        } else if (line.find("nx") != std::string::npos) {
            if (!next() || !(iss >> c->nx >> c->ny)) return bad("nx");
            nlines++;
        } else if (line.find("Lx") != std::string::npos) {
            if (!next() || !(iss >> c->lx >> c->ly)) return bad("Lx");
        } else if (line.find("w-AD") != std::string::npos) {
            // w-AD and w-PPE are ints in the reference (src/header/globalVariables.cuh:26);
            // read as numbers so that a relaxation factor such as 0.8 is kept
            double wa = 1.0, wp = 1.0;
            if (!next() || !(iss >> wa >> wp >> c->ad_itermax >> c->ppe_itermax >> c->ad_solver >> c->ppe_solver))
                return bad("w-AD");
            c->w_ad = (int)wa;
            c->w_ppe = (int)wp;
            c->relax_ad = wa;
            c->relax_ppe = wp;
        } else if (line.find("ErrorMax") != std::string::npos) {
            if (!next() || !(iss >> c->error_max >> c->tmax >> c->dt >> c->re >> c->mu)) return bad("ErrorMax");
        } else if (line.find("Write Interval") != std::string::npos) {
            if (!next() || !(iss >> c->write_interval)) return bad("Write Interval");
        // extension keywords
        } else if (line.find("Solver-Mode") != std::string::npos) {
            std::string w;
            if (!next() || !(iss >> w)) return bad("Solver-Mode");
            if (w == "reference" || w == "0") c->mode = IFX_MODE_REFERENCE;
            else if (w == "method" || w == "1") c->mode = IFX_MODE_METHOD;
            else return bad("Solver-Mode");
        } else if (line.find("Precision") != std::string::npos) {
            std::string w;
            if (!next() || !(iss >> w)) return bad("Precision");
            if (w == "fp64") c->precision = IFX_PREC_FP64;
            else if (w == "mixed") c->precision = IFX_PREC_MIXED;
            else return bad("Precision");
        } else if (line.find("Initial-Field") != std::string::npos) {
            std::string w;
            if (!next() || !(iss >> w)) return bad("Initial-Field");
            if (w == "vortex") c->init = IFX_INIT_VORTEX;
            else if (w == "uniform") c->init = IFX_INIT_UNIFORM;
            else if (w == "rest") c->init = IFX_INIT_REST;
            else return bad("Initial-Field");
        } else if (line.find("Boundary-Types") != std::string::npos) {
            std::string w[4];
            if (!next() || !(iss >> w[0] >> w[1] >> w[2] >> w[3])) return bad("Boundary-Types");
            for (int s = 0; s < 4; s++)
                if (!parse_bc(w[s], &c->bc_type[s])) return bad("Boundary-Types");
        } else if (line.find("Boundary-Velocity") != std::string::npos) {
            if (!next()) return bad("Boundary-Velocity");
            for (int s = 0; s < 4; s++)
                if (!(iss >> c->bc_u[s] >> c->bc_v[s])) return bad("Boundary-Velocity");
        } else if (line.find("Outflow-Speed") != std::string::npos) {
            if (!next() || !(iss >> c->outflow_uc)) return bad("Outflow-Speed");
        } else if (line.find("Body-Motion") != std::string::npos) {
            // none | prescribed u v amp_x amp_y amp_deg freq phase_x phase_y phase_deg
            std::string w;
            if (!next() || !(iss >> w)) return bad("Body-Motion");
            if (w == "none") {
                c->motion = IFX_MOTION_NONE;
            } else if (w == "prescribed") {
                c->motion = IFX_MOTION_PRESCRIBED;
                if (!(iss >> c->motion_u >> c->motion_v >> c->motion_amp_x >> c->motion_amp_y >> c->motion_amp_deg >>
                      c->motion_freq >> c->motion_phase_x >> c->motion_phase_y >> c->motion_phase_deg))
                    return bad("Body-Motion");
            } else {
                return bad("Body-Motion");
            }
        } else if (line.find("Body") != std::string::npos) {
            std::string w;
            if (!next() || !(iss >> w)) return bad("Body");
            if (w == "none") {
                c->body = IFX_BODY_NONE;
            } else if (w == "ellipse" || w == "circle") {
                c->body = IFX_BODY_ELLIPSE;
                if (w == "circle") {
                    double r;
                    if (!(iss >> c->body_cx >> c->body_cy >> r)) return bad("Body");
                    c->body_a = c->body_b = r;
                    c->body_angle_deg = 0.0;
                } else if (!(iss >> c->body_cx >> c->body_cy >> c->body_a >> c->body_b >> c->body_angle_deg)) {
                    return bad("Body");
                }
            } else {
                return bad("Body");
            }
        } else if (line.find("PPE-Tolerance") != std::string::npos) {
            if (!next() || !(iss >> c->ppe_tol >> c->ad_tol)) return bad("PPE-Tolerance");
        } else if (line.find("Multigrid") != std::string::npos) {
            if (!next() || !(iss >> c->mg_pre >> c->mg_post >> c->mg_omega)) return bad("Multigrid");
        } else if (line.find("Mixed-Inner") != std::string::npos) {
            if (!next() || !(iss >> c->mixed_inner)) return bad("Mixed-Inner");
        } else if (line.find("Coarse-Sweeps") != std::string::npos) {
            if (!next() || !(iss >> c->coarse_sweeps)) return bad("Coarse-Sweeps");
        } else if (line.find("Defect-Correction") != std::string::npos) {
            if (!next() || !(iss >> c->restart_drop >> c->restart_every)) return bad("Defect-Correction");
        } else if (line.find("Force-Reference") != std::string::npos) {
            if (!next() || !(iss >> c->force_ref_u >> c->force_ref_len)) return bad("Force-Reference");
        } else if (line.find("PPE-Method") != std::string::npos) {
            std::string w;
            if (!next() || !(iss >> w)) return bad("PPE-Method");
            if (w == "jacobi" || w == "0") c->ppe_method = IFX_PPE_JACOBI;
            else if (w == "point-gs" || w == "1") c->ppe_method = IFX_PPE_POINT_GS;
            else if (w == "line-sor" || w == "2") c->ppe_method = IFX_PPE_LINE_SOR;
            else return bad("PPE-Method");
        } else if (line.find("Grid-Files") != std::string::npos) {
            if (!next() || !(iss >> xg >> yg)) return bad("Grid-Files");
        }
    }
    if (c->nx < 1 || c->ny < 1) return set_error(IFX_ERR_PARSE, std::string(path) + ": nx, ny must be >= 1");
    if (IFX_PADDED_CELLS(c->nx, c->ny) > IFX_MAX_CELLS)
        return set_error(IFX_ERR_PARSE, std::string(path) + ": nx, ny give more than IFX_MAX_CELLS cells");
    const std::string d = dir_of(path);
    auto full = [&](const std::string& g) { return (!g.empty() && g[0] == '/') ? g : d + "/" + g; };
    std::snprintf(c->xgrid, IFX_PATH_MAX, "%s", full(xg).c_str());
    std::snprintf(c->ygrid, IFX_PATH_MAX, "%s", full(yg).c_str());
    (void)nlines;
    return IFX_OK;
}

// Grid-file loop of readGridData (src/include/preSim.cu:275-290): n lines of
// "<index> <coordinate>".
extern "C" ifx_status ifx_grid_read(const char* path, int n, double* coords) {
    if (!path || !coords || n < 2) return set_error(IFX_ERR_ARG, "ifx_grid_read: bad argument");
    std::ifstream f(path);
    if (!f) return set_error(IFX_ERR_IO, std::string("Error opening ") + path);
    for (int i = 0; i < n; i++) {
        long idx;
        double x;
        if (!(f >> idx >> x))
            return set_error(IFX_ERR_PARSE, std::string(path) + ": expected " + std::to_string(n) +
                                                " lines '<index> <coordinate>', got " + std::to_string(i));
        coords[i] = x;
    }
    for (int i = 1; i < n; i++)
        if (!(coords[i] > coords[i - 1]))
            return set_error(IFX_ERR_PARSE, std::string(path) + ": coordinates must increase");
    return IFX_OK;
}

// write_results_to_file (src/include/postSim.cu:41-66), byte for byte.
extern "C" ifx_status ifx_write_tecplot(const char* path, int nx, int ny, const double* x, const double* y,
                                        const double* q) {
    if (!path || !x || !y || !q || nx < 1 || ny < 1) return set_error(IFX_ERR_ARG, "ifx_write_tecplot: bad argument");
    FILE* fp = std::fopen(path, "w");
    if (!fp) return set_error(IFX_ERR_IO, std::string("Error opening file: ") + path);
    std::fprintf(fp, "TITLE = \"Post Processing Tecplot\"\n");
    std::fprintf(fp, "VARIABLES = \"X\",\"Y\",\"T\"\n");
    std::fprintf(fp, "ZONE T=\"BIG ZONE\", I=%d, J=%d, DATAPACKING=POINT\n", nx, ny);
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) std::fprintf(fp, "%f,%f,%f\n", x[i], y[j], q[i + (size_t)j * nx]);
    if (std::fclose(fp) != 0) return set_error(IFX_ERR_IO, std::string("Error closing file: ") + path);
    return IFX_OK;
}
