// Host side of the reference class surface: Engine (device context), elliptic / hyperbolic
// solver classes, the Impec2DSolver time loop with its diagnostics and output files, the
// well initialisers and the reference's two convergence tests, all calling the C ABI.
#include <cuda_runtime.h>
#include <sys/stat.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>

#include "Solvers.h"

namespace impec {
void set_error(const std::string& msg);  // the library's last-error record (impec_last_error)
}

// ---------------------------------------------------------------- host ghost fills
// Reflection form of FillGhostCellsNeumannScalar / FillGhostCellsPeriodicScalar /
// FillGhostCellsNeumannVelocity (src/Util.cpp:215-438).
static int rcell(int i, int n) { return i < 0 ? -1 - i : (i >= n ? 2 * n - 1 - i : i); }
static int wcell(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

void FillGhostCellsNeumannScalar(Array2d& a, int N1, int N2, int g) {
    for (int i = -g; i < N1 + g; ++i)
        for (int j = -g; j < N2 + g; ++j)
            if (i < 0 || i >= N1 || j < 0 || j >= N2) a(i, j) = a(rcell(i, N1), rcell(j, N2));
}
void FillGhostCellsPeriodicScalar(Array2d& a, int N1, int N2, int g) {
    for (int i = -g; i < N1 + g; ++i)
        for (int j = -g; j < N2 + g; ++j)
            if (i < 0 || i >= N1 || j < 0 || j >= N2) a(i, j) = a(wcell(i, N1), wcell(j, N2));
}
void FillGhostCellsNeumannVelocity(Array3d& v, int N1, int N2, int g) {
    auto rf = [](int f, int n, double& s) {
        if (f < 0) { s = -s; return -f; }
        if (f > n) { s = -s; return 2 * n - f; }
        return f;
    };
    for (int i = -g; i <= N1 + g; ++i)  // u: odd in x (faces), even in y (cells)
        for (int j = -g; j < N2 + g; ++j) {
            if (i >= 0 && i <= N1 && j >= 0 && j < N2) continue;
            double s = 1.0;
            int fi = rf(i, N1, s);
            v(i, j, 0) = s * v(fi, rcell(j, N2), 0);
        }
    for (int i = -g; i < N1 + g; ++i)  // v: even in x (cells), odd in y (faces)
        for (int j = -g; j <= N2 + g; ++j) {
            if (i >= 0 && i < N1 && j >= 0 && j <= N2) continue;
            double s = 1.0;
            int fj = rf(j, N2, s);
            v(i, j, 1) = s * v(rcell(i, N1), fj, 1);
        }
}

// ---------------------------------------------------------------- Engine
Engine::Engine(const SimParams& sp) : N1(sp.N1), N2(sp.N2), g(sp.p_bounds) {
    impec_params P = sp.engine();
    check(impec_ctx_create(&P, nullptr, &ctx_), "impec_ctx_create");
    try {
        check(impec_state(ctx_, &c, &p, &u, &v, &q), "impec_state");
        check(impec_set_time(ctx_, sp.tstart), "impec_set_time");
        if (!sp.learned_weights.empty()) attach_learned(sp);
    } catch (...) {
        if (net_) impec_learned_attach(ctx_, nullptr, 1, 0), impec_net_destroy(net_);
        impec_ctx_destroy(ctx_);
        throw;
    }
}
Engine::~Engine() {
    if (net_) {
        impec_learned_attach(ctx_, nullptr, 1, 0);
        impec_net_destroy(net_);
    }
    impec_ctx_destroy(ctx_);
}

// A 1-D little-endian float32 .npy array (format versions 1-3, C order).
static std::vector<float> read_npy_f32(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw ConfigError("gb300.learned_weights: cannot open " + path);
    char magic[6];
    unsigned char ver[2];
    f.read(magic, 6);
    f.read(reinterpret_cast<char*>(ver), 2);
    if (!f || std::string(magic, 6) != "\x93NUMPY") throw ConfigError(path + ": not an .npy file");
    uint32_t hlen = 0;
    unsigned char b[4] = {0, 0, 0, 0};
    f.read(reinterpret_cast<char*>(b), ver[0] == 1 ? 2 : 4);
    hlen = b[0] | (b[1] << 8) | (ver[0] == 1 ? 0u : ((uint32_t)b[2] << 16) | ((uint32_t)b[3] << 24));
    std::string h(hlen, ' ');
    f.read(&h[0], hlen);
    auto has = [&](const char* t) { return h.find(t) != std::string::npos; };
    if (!f || !has("'descr': '<f4'") || !has("'fortran_order': False"))
        throw ConfigError(path + ": expected a little-endian float32 array in C order");
    const size_t lp = h.find("'shape': ("), rp = lp == std::string::npos ? lp : h.find(')', lp);
    if (rp == std::string::npos) throw ConfigError(path + ": no shape in the .npy header");
    const std::string shape = h.substr(lp + 10, rp - lp - 10);
    if (shape.find(',') != shape.rfind(',') || shape.find_first_not_of("0123456789, ") != std::string::npos)
        throw ConfigError(path + ": expected a 1-D array");
    const size_t n = std::stoull(shape);
    std::vector<float> w(n);
    f.read(reinterpret_cast<char*>(w.data()), (std::streamsize)(n * sizeof(float)));
    if (!f) throw ConfigError(path + ": truncated");
    return w;
}

// gb300.learned_weights: the trained network as the initial guess of every pressure solve.
void Engine::attach_learned(const SimParams& sp) {
    std::vector<float> w = read_npy_f32(sp.learned_weights);
    check(impec_net_create(0, &net_), "impec_net_create");
    size_t count = 0;
    check(impec_net_parameters(net_, nullptr, nullptr, &count, 0), "impec_net_parameters");
    if (w.size() != count)
        throw ConfigError(sp.learned_weights + ": " + std::to_string(w.size()) + " parameters, the network has " +
                          std::to_string(count));
    check(impec_net_parameters(net_, nullptr, w.data(), &count, 0), "impec_net_parameters");
    int f = sp.learned_factor;
    if (f == 0)
        for (f = 16; f > 1 && (N1 / f < 256 || N1 % (8 * f) || N2 % (8 * f)); f /= 2) {}
    check(impec_learned_attach(ctx_, net_, f, 1), "impec_learned_attach");
}
void Engine::check(impec_status s, const char* what) const {
    if (s != IMPEC_OK) throw EngineError(s, std::string(what) + ": " + impec_last_error());
}
void Engine::put_c(const Array2d& a) { check(impec_state_upload(ctx_, a.data(), nullptr, g), "upload c"); }
void Engine::get_c(Array2d& a) { check(impec_state_download(ctx_, a.data(), nullptr, nullptr, g), "download c"); }
void Engine::get_p(Array2d& a) { check(impec_state_download(ctx_, nullptr, a.data(), nullptr, g), "download p"); }
void Engine::put_v(const Array3d& a) { check(impec_velocity_upload(ctx_, a.data(), g), "upload v"); }
void Engine::get_v(Array3d& a) { check(impec_state_download(ctx_, nullptr, nullptr, a.data(), g), "download v"); }
void Engine::put_q(const double* qh) {
    // reuse the host layout entry point with a ghost-free view of q
    check(impec_state_upload(ctx_, nullptr, qh, g), "upload q");
}

void Engine::project_diagonal(int field, int dN1, int dN2, Array2d& a, int bounds) {
    std::vector<double> h((size_t)dN1 * dN2);
    check(impec_project_diagonal_download(ctx_, field, h.data(), dN1, dN2), "project_diagonal");
    a.resize(dN1 + 2 * bounds, dN2 + 2 * bounds, -bounds, -bounds);
    std::fill(a.data(), a.data() + (size_t)(dN1 + 2 * bounds) * (dN2 + 2 * bounds), 0.0);
    for (int i = 0; i < dN1; ++i)
        for (int j = 0; j < dN2; ++j) a(i, j) = h[(size_t)i * dN2 + j];
}

// ---------------------------------------------------------------- elliptic
EllipticSolver::EllipticSolver(SimParams* sp, Engine* eng) : sp(sp), eng(eng) { SetNu(sp->nu); }

void EllipticSolver::SetNu(double n) {  // src/EllipticSolver.cpp:526-534
    if (!(n >= 0. && n <= 1.)) throw ConfigError("EllipticSolver::SetNu> Invalid value for nu");
    nu = n;
}

bool EllipticSolver::Solve(Array2d& p, Array2d& c, double* q) {  // src/EllipticSolver.cpp:133-142
    calls++;
    bool ret = SolveLinearMultigrid(c, sp->c_bounds, p, sp->p_bounds, q);
    total_its += last_its;
    return ret;
}

void EllipticSolver::CalcVelocities(Array2d& p, Array3d& v, Array2d& c) {  // src/EllipticSolver.cpp:660-683
    FillGhostCellsNeumannScalar(p, sp->N1, sp->N2, sp->p_bounds);
    eng->put_c(c);
    eng->check(impec_pressure_upload(eng->ctx(), p.data(), sp->p_bounds), "upload p");
    eng->check(impec_velocity(eng->ctx(), eng->p, eng->c, eng->u, eng->v), "impec_velocity");
    eng->get_v(v);
    FillGhostCellsNeumannVelocity(v, sp->N1, sp->N2, sp->v_bounds);
}

bool MGSolver::SolveLinearMultigrid(Array2d& c, int c_bounds, Array2d& p, int, const double* q) {
    if (c_bounds <= 0) return false;  // src/MGSolver.cpp:224-227
    eng->put_c(c);
    eng->put_q(q);
    int cyc = 0;
    impec_status s = impec_pressure_solve(eng->ctx(), eng->c, eng->p, sp->eps, &cyc, &last_relres);
    last_its = cyc;
    if (s != IMPEC_OK && s != IMPEC_ERR_NOT_CONVERGED) eng->check(s, "impec_pressure_solve");
    eng->get_p(p);
    return s == IMPEC_OK;
}

bool MGSolver::Solve_Parabolic_cc_to_c(Array2d& c, int, const Array3d& v, int, double dt) {
    eng->put_c(c);
    eng->put_v(v);
    int its = 0;
    double rr = 0;
    impec_status s = impec_dispersion_cn(eng->ctx(), eng->c, eng->u, eng->v, dt, sp->para_eps, &its, &rr);
    last_parabolic_its = its;
    eng->get_c(c);
    return s == IMPEC_OK;
}

// ---------------------------------------------------------------- hyperbolic
int TRIntegrator::Integrate(Array2d& c, const double* q, double dt) {  // src/TRIntegrator.cpp:49-71
    eng->put_c(c);
    eng->put_q(q);
    eng->check(impec_tr_integrate(eng->ctx(), eng->c, dt, &total_mass_outflux), "impec_tr_integrate");
    eng->get_c(c);
    return 0;
}

void HyperbolicSolver::FillBoundaries(Array2d& c) {  // src/HyperbolicSolver.cpp:56-61
    if (sp->is_test) FillGhostCellsPeriodicScalar(c, sp->N1, sp->N2, sp->c_bounds);
    else FillGhostCellsNeumannScalar(c, sp->N1, sp->N2, sp->c_bounds);
}

double HyperbolicSolver::MaxStableTimestep(const Array2d&, const Array3d& v) {
    if (sp->is_test) {  // MaxStableAdvectionTimestep (src/HyperbolicSolver.cpp:96-121)
        double dtm = 1e300;
        const double tiny = 2.2250738585072014e-308;
        for (int i = 0; i < sp->N1; ++i)
            for (int j = 0; j < sp->N2; ++j) {
                double uc = std::max(std::fabs(0.5 * (v(i, j, 0) + v(i + 1, j, 0))), tiny);
                double vc = std::max(std::fabs(0.5 * (v(i, j, 1) + v(i, j + 1, 1))), tiny);
                dtm = std::min(dtm, std::min(sp->dx / uc, sp->dy / vc));
            }
        return dtm * sp->cfl;
    }
    eng->put_v(v);
    double dt = 0;
    eng->check(impec_max_stable_dt(eng->ctx(), eng->u, eng->v, &dt), "impec_max_stable_dt");
    return dt;
}

bool HyperbolicSolver::SourceSplit(Array2d& c, const double* q, double dt) {  // :201-205
    ti.Integrate(c, q, dt);
    total_mass_outflux += std::fabs(ti.GetTotalMassOutflux());
    return true;
}

bool HyperbolicSolver::DiffusionSplit(Array2d& c, const Array3d& v, double dt) {  // :213-223
    if (!mg) throw EngineError(IMPEC_ERR_ARG, "HyperbolicSolver:: a multigrid solver is needed for Crank-Nicolson");
    return mg->Solve_Parabolic_cc_to_c(c, sp->c_bounds, v, sp->v_bounds, dt);
}

bool HyperbolicSplitSolver::Advect_X(Array2d& c, const Array3d& v, double dt) {
    eng->put_c(c);
    eng->put_v(v);
    eng->check(impec_advect_x(eng->ctx(), eng->c, eng->u, dt), "impec_advect_x");
    eng->get_c(c);
    return true;
}

bool HyperbolicSplitSolver::Advect_Y(Array2d& c, const Array3d& v, double dt) {
    eng->put_c(c);
    eng->put_v(v);
    eng->check(impec_advect_y(eng->ctx(), eng->c, eng->v, dt), "impec_advect_y");
    eng->get_c(c);
    return true;
}

bool HyperbolicSplitSolver::AdvectSplit(Array2d& c, const Array3d& v, const double*, double dt) {
    eng->put_c(c);
    eng->put_v(v);
    int pfs = prev_first_sweep == X_SWEEP ? 0 : 1;
    eng->check(impec_advect_split(eng->ctx(), eng->c, eng->u, eng->v, dt, &pfs), "impec_advect_split");
    prev_first_sweep = pfs == 0 ? X_SWEEP : Y_SWEEP;
    eng->get_c(c);
    return true;
}

bool HyperbolicSplitSolver::Solve(Array2d& c, const Array3d& v, const double* q, double dt) {
    eng->put_c(c);
    eng->put_v(v);
    eng->put_q(q);
    int pfs = prev_first_sweep == X_SWEEP ? 0 : 1;
    double of = total_mass_outflux;
    eng->check(impec_hyperbolic_solve(eng->ctx(), eng->c, eng->u, eng->v, dt, &pfs, &of), "impec_hyperbolic_solve");
    total_mass_outflux = of;
    prev_first_sweep = pfs == 0 ? X_SWEEP : Y_SWEEP;
    eng->get_c(c);
    FillBoundaries(c);
    return true;
}

// ---------------------------------------------------------------- wells (src/Util.cpp:444-639)
static double ExactVolFracCircle(double x1, double y1, double r, double dx, double dy) {
    if (!(x1 * x1 + y1 * y1 < r * r)) return 0;
    double y2 = y1 + dy, x2 = x1 + dx;
    if (!(x2 * x2 + y2 * y2 > r * r)) return 1.;
    double xs = std::sqrt(r * r - y1 * y1), ys = std::sqrt(r * r - x1 * x1);
    double area = 0, xub, xlb;
    if (ys <= y2 && xs <= x2) {
        xlb = x1; xub = xs;
    } else if (ys < y2 && xs > x2) {
        xlb = x1; xub = x2;
    } else if (ys > y2 && xs < x2) {
        xlb = std::sqrt(r * r - y2 * y2); xub = xs;
        area += (xlb - x1) * dy;
    } else {
        xlb = std::sqrt(r * r - y2 * y2); xub = x2;
        area += dy * (xlb - x1);
    }
    double t1 = std::asin(xlb / r), t2 = std::asin(xub / r);
    area += r * r / 2 * (std::sin(2 * t2) / 2. + t2 - std::sin(2 * t1) / 2. - t1);
    area -= y1 * (xub - xlb);
    return area / (dx * dy);
}

void InitializeSourceTerm(const SimParams& sp, double* q, double t) {
    const int N1 = sp.N1, N2 = sp.N2, M = N1 * N2;
    const double dx = sp.dx, dy = sp.dy;
    std::fill(q, q + M, 0.0);
    if (sp.stype == HORIZONTAL) {  // InitHorizontalFront :607-639
        int w = (int)std::lround(sp.well_width * (sp.x_ub - sp.x_lb) / dx);
        if (w < 1) throw ConfigError("Injection layer cannot be represented on this grid: (qlayer_width < 1)");
        double val = sp.I / (N2 * dx * dy * w);
        if (sp.im == PULSING) {
            double tau = 1. / sp.q_freq;
            if (std::fmod(t, tau) > tau / 2.) val *= sp.q_high_multiple;
        } else if (sp.im == LINEAR) {
            double vl = val, vh = val * sp.q_high_multiple;
            val = vl + (t - sp.tstart) * (vh - vl) / (sp.tfinal - sp.tstart);
        }
        for (int i = 0; i < N2 * w; i++) {
            q[i] = val;
            q[M - 1 - i] = -val;
        }
        return;
    }
    const double qval = sp.I / (dx * dy);
    if (sp.well_profile == ONECELL) {
        q[0] = qval;
        if (sp.stype == PARALLEL) {
            q[M - 1] = qval;
            q[N2 - 1] = -qval;
            q[(N1 - 1) * N2] = -qval;
        } else {
            q[M - 1] = -qval;
        }
    } else if (sp.well_profile == CIRCULAR) {
        double r = sp.well_rc * (sp.x_ub - sp.x_lb);
        double cv = sp.I * 4. / (M_PI * r * r);
        std::vector<double> I((size_t)M);
        for (int i = 0; i < N1; ++i)
            for (int j = 0; j < N2; ++j)
                I[(size_t)i * N2 + j] = cv * ExactVolFracCircle(sp.x_lb + i * dx, sp.y_lb + j * dy, r, dx, dy);
        auto at = [&](int i, int j) { return I[(size_t)i * N2 + j]; };
        for (int i = 0; i < N1; ++i)
            for (int j = 0; j < N2; ++j)
                q[(size_t)i * N2 + j] = sp.stype == DIAGONAL
                                            ? at(i, j) - at(N1 - 1 - i, N2 - 1 - j)
                                            : at(i, j) + at(N1 - 1 - i, N2 - 1 - j) - at(i, N2 - 1 - j) - at(N1 - 1 - i, j);
    }
}

// ---------------------------------------------------------------- output (src/Printer.cpp)
void PrintDToPlotFile(const std::string& fn, const Array2d& a, double x_lb, double y_lb, double dx, double dy, int sb) {
    std::ofstream f(fn);
    if (!f) {
        std::cerr << "PRINTER-ERROR: Unable to write to file: " << fn << std::endl;
        return;
    }
    const int sx = a.base(0) + sb, sy = a.base(1) + sb, ex = sx + a.extent(0) - 2 * sb, ey = sy + a.extent(1) - 2 * sb;
    for (int i = sx; i < ex; i++) {
        for (int j = sy; j < ey; j++) f << x_lb + (i + 0.5) * dx << " " << y_lb + (j + 0.5) * dy << " " << a(i, j) << "\n";
        f << "\n";
    }
}

void PrintVelToPlotFile(const std::string& uf, const std::string& vf, const Array3d& a, double x_lb, double y_lb,
                        double dx, double dy, int sb) {
    std::ofstream fu(uf), fv(vf);
    if (!fu || !fv) {
        std::cerr << "PRINTER-ERROR: Unable to write to file: " << uf << " or " << vf << std::endl;
        return;
    }
    const int sx = a.base(0) + sb, sy = a.base(1) + sb, ex = sx + a.extent(0) - 2 * sb, ey = sy + a.extent(1) - 2 * sb;
    for (int i = sx; i < ex; i++) {
        for (int j = sy; j < ey - 1; j++) fu << x_lb + i * dx << " " << y_lb + (j + 0.5) * dy << " " << a(i, j, 0) << "\n";
        fu << "\n";
    }
    for (int i = sx; i < ex - 1; i++) {
        for (int j = sy; j < ey; j++) fv << x_lb + (i + 0.5) * dx << " " << y_lb + j * dy << " " << a(i, j, 1) << "\n";
        fv << "\n";
    }
}

// ---------------------------------------------------------------- Impec2DSolver
static void ensure_dir(const std::string& d) {
    struct stat st;
    if (d.empty() || stat(d.c_str(), &st) == 0) return;
    if (mkdir(d.c_str(), 0755) != 0) throw ConfigError("Error: could not create " + d);
}

Impec2DSolver::Impec2DSolver(const std::string& cfgfile, int myid, int nprocs) : myid(myid), num_procs(nprocs) {
    sp = new SimParams(cfgfile);
    Initialize();
}

Impec2DSolver::~Impec2DSolver() {
    delete hs;
    delete es;
    delete eng;
    delete sp;
}

void Impec2DSolver::Initialize() {  // src/Impec2DSolver.cpp:125-143
    if (sp->is_test) return;  // tests build their own grids
    if (sp->log_to_file) ensure_dir(sp->log_dir);
    ensure_dir(sp->results_dir);
    eng = new Engine(*sp);
    MGSolver* mg = new MGSolver(sp, eng);
    es = mg;
    if (sp->hmtype == UPWINDSPLIT) hs = new UpwindSplitSolver(sp, eng);
    else hs = new MUSCLSplitSolver(sp, eng);
    hs->AssignMGSolver(mg);
    ResizeArrays();
    InitializeConcentration();
    InitializeSource();
}

void Impec2DSolver::ResizeArrays() {  // src/Impec2DSolver.cpp:151-182
    const int g = sp->p_bounds;
    p.resize(sp->N1 + 2 * g, sp->N2 + 2 * g, -g, -g);
    c.resize(sp->N1 + 2 * g, sp->N2 + 2 * g, -g, -g);
    v.resize(sp->N1 + 1 + 2 * g, sp->N2 + 1 + 2 * g, 2, -g, -g);
    q.assign((size_t)sp->M, 0.0);
}

void Impec2DSolver::InitializeConcentration() {  // src/Impec2DSolver.cpp:191-233
    c = 0.0;
    if (sp->init_file.empty()) return;
    std::ifstream f(sp->init_file);
    if (!f) {
        std::cout << "Unable to open file" << sp->init_file << "; Initializing to zero." << std::endl;
        return;
    }
    std::string line;
    int ctr = 0;
    while (std::getline(f, line)) {
        if (line.empty()) continue;
        std::stringstream ss(line);
        double x, y, conc;
        if (!(ss >> x >> y >> conc)) continue;
        if (ctr >= sp->N1 * sp->N2) throw ConfigError("Concentration Input FILE:: wrong dimensions!");
        c(ctr / sp->N2, ctr % sp->N2) = conc;
        ctr++;
    }
    if (ctr != sp->N1 * sp->N2) throw ConfigError("Concentration Input FILE:: wrong dimensions!");
}

void Impec2DSolver::InitializeSource() { InitializeSourceTerm(*sp, q.data(), sp->tstart); }

double Impec2DSolver::CalculateMassError(double t, double mass) {  // :530-540
    double influx = (t - sp->tstart) * sp->I * (1. / (sp->dx * sp->dy));
    if (sp->stype == PARALLEL) influx *= 2.;
    return std::fabs((mass + hs->GetTotalMassOutflux() - influx) / influx);
}

void Impec2DSolver::WriteDiagnostics(const std::vector<DiagState>& ds) {  // :469-494
    std::string fn = sp->results_dir + "/diagnostics.dat";
    std::ofstream f(fn);
    if (!f) {
        std::cerr << "Unable to write to diagnostics-file: " << fn << std::endl;
        return;
    }
    const std::string SEP = "    ";
    for (const DiagState& d : ds) {
        f << d.ctr << SEP << d.its << SEP << d.t << SEP << d.dt << SEP << d.fillperdt << SEP;
        if (sp->check_mass_conservation) f << d.mass_err << SEP;
        if (sp->check_noflow_boundary) f << d.vel_err << SEP;
        if (sp->check_divergence) f << d.diff_err << SEP;
        f << "\n";
    }
}

void Impec2DSolver::LogResults(const std::string& postfix) {  // LogResultsMatch :622-686
    const bool final = postfix.empty();
    const std::string dir = final ? sp->results_dir : sp->log_dir;
    const std::string sfx = final ? ".dat" : postfix + ".dat";
    if (sp->stype == PARALLEL) {
        // parallel runs are written on the diagonal grid (Project, src/Impec2DSolver.cpp:645-666, 690-716)
        const int dN1 = (int)std::lround(sp->N1 / std::sqrt(2.)), dN2 = (int)std::lround(sp->N2 / std::sqrt(2.));
        const double d_dx = (sp->x_ub - sp->x_lb) / (std::sqrt(2.) * dN1);
        const double d_dy = (sp->y_ub - sp->y_lb) / (std::sqrt(2.) * dN2);
        Array2d diag;
        eng->project_diagonal(0, dN1, dN2, diag, sp->c_bounds);
        PrintDToPlotFile(dir + "/concentration" + sfx, diag, sp->x_lb, sp->y_lb, d_dx, d_dy, sp->c_bounds);
        if (final) {
            eng->project_diagonal(1, dN1, dN2, diag, sp->p_bounds);
            PrintDToPlotFile(dir + "/pressure" + sfx, diag, sp->x_lb, sp->y_lb, d_dx, d_dy, sp->p_bounds);
        }
        return;
    }
    eng->get_c(c);
    PrintDToPlotFile(dir + "/concentration" + sfx, c, sp->x_lb, sp->y_lb, sp->dx, sp->dy, sp->c_bounds);
    if (final) {
        eng->get_p(p);
        eng->get_v(v);
        PrintDToPlotFile(dir + "/pressure" + sfx, p, sp->x_lb, sp->y_lb, sp->dx, sp->dy, sp->p_bounds);
        PrintVelToPlotFile(dir + "/velocity_u" + sfx, dir + "/velocity_v" + sfx, v, sp->x_lb, sp->y_lb, sp->dx, sp->dy,
                           sp->v_bounds);
    }
}

bool Impec2DSolver::Solve(bool quiet) {  // src/Impec2DSolver.cpp:293-466, resident state
    auto t_start = std::chrono::steady_clock::now();
    std::vector<double> times = sp->times;
    if (std::find(times.begin(), times.end(), sp->tfinal) == times.end()) times.push_back(sp->tfinal);
    std::sort(times.begin(), times.end());
    size_t tidx = 0;
    eng->put_c(c);
    eng->put_q(q.data());
    eng->check(impec_set_time(eng->ctx(), sp->tstart), "impec_set_time");
    double t = sp->tstart, maxc = 0, minc = 10e10, avg_fill = 0;
    int counter = 0, total_its = 0;
    bool state = true;
    if (!quiet) std::cout << "Final time: " << sp->tfinal << std::endl;
    diag.clear();
    while (state && t < sp->tfinal) {
        counter++;
        impec_step_info info;
        double t_clip = tidx < times.size() ? times[tidx] : -1.0;
        impec_status s = impec_step(eng->ctx(), t_clip, &info);
        if (s != IMPEC_OK) {
            std::cerr << "ERROR::Impec2DSolver: [" << counter << "]\tt:\t" << t << "\t" << impec_last_error() << std::endl;
            state = false;
            break;
        }
        if (info.clipped) tidx++;
        t = info.t;
        total_its += info.its;
        DiagState ds{};
        ds.ctr = counter;
        ds.t = t;
        ds.dt = info.dt;
        ds.its = info.its;
        ds.fillperdt = info.dt * sp->I / (sp->dx * sp->dy);
        avg_fill += ds.fillperdt;
        double d5[5] = {0, 0, 0, 0, 0};
        eng->check(impec_diagnostics(eng->ctx(), eng->c, eng->u, eng->v, d5), "impec_diagnostics");
        double influx = (t - sp->tstart) * sp->I * (1. / (sp->dx * sp->dy)) * (sp->stype == PARALLEL ? 2. : 1.);
        ds.mass_err = sp->check_mass_conservation ? std::fabs((d5[0] + info.total_outflux - influx) / influx) : -1;
        ds.vel_err = sp->check_noflow_boundary ? d5[2] : -1;
        ds.diff_err = sp->check_divergence ? d5[1] : -1;
        maxc = std::max(maxc, d5[3]);
        minc = std::min(minc, d5[4]);
        diag.push_back(ds);
        if (!quiet && myid == 0) {  // OutputState :499-527
            std::ostringstream ss;
            ss.setf(std::ios_base::fixed, std::ios_base::floatfield);
            ss.precision(6);
            ss << "[" << ds.ctr << "]\tITS_e: " << ds.its << "\tITS_p: " << info.para_its << "\t t: " << ds.t
               << "\tdt: " << ds.dt << "\tcells/dt: " << ds.fillperdt;
            if (sp->check_mass_conservation) ss << "\tE_m: " << ds.mass_err * 100;
            if (sp->check_noflow_boundary) ss << "\tE_v: " << ds.vel_err;
            if (sp->check_divergence) ss << "\tE_div: " << ds.diff_err;
            std::cout << ss.str() << std::endl;
        }
        if (sp->log_to_file && myid == 0) {
            bool is_time = std::find(sp->times.begin(), sp->times.end(), t) != sp->times.end();
            if (is_time) {
                std::ostringstream pf;
                pf << "_t_" << t;
                LogResults(pf.str());
            }
            bool is_step = std::find(sp->counters.begin(), sp->counters.end(), counter) != sp->counters.end();
            if (is_step || (sp->log_skip_steps != 0 && (counter == 1 || counter % sp->log_skip_steps == 0)))
                LogResults("_" + std::to_string(counter));
        }
        if (sp->stype == HORIZONTAL && sp->im != CONSTANT) {  // src/Impec2DSolver.cpp:437-439
            InitializeSourceTerm(*sp, q.data(), t);
            eng->put_q(q.data());  // same well cells: the step graph is kept, only the rates change
        }
    }
    if (counter > 0) avg_fill /= counter;
    if (myid == 0) {
        long ms = (long)std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
        if (!quiet) {
            std::cout << "overall maximum: " << maxc << "\noverall minimum: " << minc
                      << "\naverage filled cells per dt: " << avg_fill << std::endl;
            std::cout << "---------------------------------------------------------" << std::endl;
            if (counter > 0) std::cout << "Average no. of Iterations: " << (double)total_its / counter << std::endl;
            std::cout << "Elapsed time [ms]: " << ms << std::endl;
        }
        LogResults("");
        WriteDiagnostics(diag);
    }
    return state;
}

bool Impec2DSolver::Run() { return sp->is_test ? TestComponent() : Solve(false); }

// TestComponent -> TestNeumann / TestAdvection (src/Impec2DSolver.cpp:719-1015,
// src/EllipticSolver.cpp:155-470), run through the engine.
bool Impec2DSolver::TestComponent() {
    std::ofstream norm(sp->norm_file);
    if (!norm) {
        std::cerr << "Cannot write norm-file! Convergence test aborted..." << std::endl;
        return false;
    }
    norm.precision(30);
    int N1 = sp->init_x_cells, N2 = sp->init_y_cells;
    for (int k = 0; k < sp->levels; ++k, N1 *= 2, N2 *= 2) {
        SimParams s = *sp;
        s.N1 = N1; s.N2 = N2; s.M = N1 * N2;
        s.dx = (s.x_ub - s.x_lb) / N1;
        s.dy = (s.y_ub - s.y_lb) / N2;
        const int g = s.p_bounds;
        Engine E(s);
        std::cout << "-> (N1,N2):\t(" << N1 << " , " << N2 << ")";
        if (s.test_component == ELLIPTIC) {
            impec_params P = s.engine();
            const double t2 = 2.;
            auto K11 = [&](double x, double y) {
                switch (s.testno) { case 2: return std::exp(-0.3 * x); case 3: case 4: return 2. + std::sin(t2 * x) * std::sin(y); default: return 1.; }
            };
            auto K22 = [&](double x, double y) {
                switch (s.testno) { case 2: return std::exp(-0.3 * y); case 3: return 2. + std::sin(t2 * x) * std::sin(y); case 4: return 2. + std::sin(x) * std::sin(t2 * y); default: return 1.; }
            };
            auto qT = [&](double x, double y) {
                double a1 = K11(x, y), a2 = K22(x, y), a1x = 0, a2y = 0;
                switch (s.testno) {
                    case 2: a1x = -0.3 * std::exp(-0.3 * x); a2y = -0.3 * std::exp(-0.3 * y); break;
                    case 3: a1x = t2 * std::cos(t2 * x) * std::sin(y); a2y = std::cos(y) * std::sin(t2 * x); break;
                    case 4: a1x = t2 * std::cos(t2 * x) * std::sin(y); a2y = t2 * std::cos(t2 * y) * std::sin(x); break;
                    default: a1 = a2 = 1.; break;
                }
                return 1. / s.mu_res * ((a1 + a2) * std::cos(x) * std::cos(y) + a1x * std::sin(x) * std::cos(y) + a2y * std::cos(x) * std::sin(y));
            };
            std::vector<double> k1((size_t)N1 * N2), k2((size_t)N1 * N2), qq((size_t)N1 * N2);
            for (int i = 0; i < N1; ++i)
                for (int j = 0; j < N2; ++j) {
                    double x = s.x_lb + (i + 0.5) * s.dx, y = s.y_lb + (j + 0.5) * s.dy;
                    k1[(size_t)i * N2 + j] = K11(x, y);
                    k2[(size_t)i * N2 + j] = K22(x, y);
                    qq[(size_t)i * N2 + j] = qT(x, y);
                }
            (void)P;
            double *dk1, *dk2;
            cudaMalloc((void**)&dk1, k1.size() * 8);
            cudaMalloc((void**)&dk2, k2.size() * 8);
            cudaMemcpy(dk1, k1.data(), k1.size() * 8, cudaMemcpyHostToDevice);
            cudaMemcpy(dk2, k2.data(), k2.size() * 8, cudaMemcpyHostToDevice);
            E.check(impec_set_permeability(E.ctx(), dk1, dk2), "impec_set_permeability");
            cudaFree(dk1);
            cudaFree(dk2);
            double xp = s.x_lb + 1.5 * s.dx, yp = s.y_lb + 1.5 * s.dy;  // pinned cell (1,1), :527-548
            E.check(impec_set_pin_kappa(E.ctx(), -s.dx * s.dy * qT(xp, yp) / (std::cos(xp) * std::cos(yp))), "pin");
            E.put_q(qq.data());
            Array2d c0(N1 + 2 * g, N2 + 2 * g, -g, -g), pp(N1 + 2 * g, N2 + 2 * g, -g, -g);
            Array3d vv;
            vv.resize(N1 + 1 + 2 * g, N2 + 1 + 2 * g, 2, -g, -g);
            E.put_c(c0);
            int cyc = 0;
            double rr = 0;
            E.check(impec_pressure_solve(E.ctx(), E.c, E.p, s.eps, &cyc, &rr), "impec_pressure_solve");
            E.check(impec_velocity(E.ctx(), E.p, E.c, E.u, E.v), "impec_velocity");
            E.get_p(pp);
            E.get_v(vv);
            std::cout << "\tITS:\t" << cyc << std::endl;
            double ps = 0, us = 0, vs = 0;
            for (int i = 0; i < N1; i++)
                for (int j = 0; j < N2; j++) {
                    double x = s.x_lb + (i + 0.5) * s.dx, y = s.y_lb + (j + 0.5) * s.dy;
                    ps += std::fabs(pp(i, j) - std::cos(x) * std::cos(y));
                }
            for (int i = 0; i <= N1; i++)
                for (int j = 0; j < N2; j++) {
                    double x = s.x_lb + i * s.dx, y = s.y_lb + (j + 0.5) * s.dy;
                    us += std::fabs(K11(x, y) / s.mu_res * std::sin(x) * std::cos(y) - vv(i, j, 0));
                }
            for (int i = 0; i < N1; i++)
                for (int j = 0; j <= N2; j++) {
                    double x = s.x_lb + (i + 0.5) * s.dx, y = s.y_lb + j * s.dy;
                    vs += std::fabs(K22(x, y) / s.mu_res * std::cos(x) * std::sin(y) - vv(i, j, 1));
                }
            double dA = s.dx * s.dy;
            norm << std::log(s.dx) << "\t" << std::log(ps * dA) << "\t" << std::log(us * dA) << "\t" << std::log(vs * dA) << "\n";
        } else {  // hyperbolic: Advection (src/Impec2DSolver.cpp:848-990)
            const double L = s.x_ub - s.x_lb, H = s.y_ub - s.y_lb;
            Array2d cc(N1 + 2 * g, N2 + 2 * g, -g, -g);
            auto prof = [&](double x, double y) {
                const double dx = s.dx, dy = s.dy, xc = L / 2., yc = H / 2.;
                switch (s.hyp_test) {
                    case SINE: return 1. + 1. / (dx * dy * 4. * M_PI * M_PI) * (std::cos(2. * M_PI * (x + dx / 2.)) - std::cos(2. * M_PI * (x - dx / 2.))) *
                                               (std::cos(2. * M_PI * (y + dy / 2.)) - std::cos(2. * M_PI * (y - dy / 2.)));
                    case TOPHAT: return (std::fabs(x - xc) <= 0.3 * L / 2. && std::fabs(y - yc) <= 0.3 * H / 2.) ? 1. : 0.;
                    case GAUSS: {
                        double ix = 1. / 16 * std::sqrt(M_PI) * (-std::erf(8. * xc - 4. * dx - 8. * x) + std::erf(8. * xc + 4. * dx - 8. * x));
                        double iy = 1. / 16 * std::sqrt(M_PI) * (-std::erf(8. * yc - 4. * dy - 8. * y) + std::erf(8. * yc + 4. * dy - 8. * y));
                        return 1. / (dx * dy) * ix * iy;
                    }
                    default: return 1. + 1. / dy * (-1. / (2. * M_PI)) * (std::cos(2 * M_PI * (y + dy / 2.)) - std::cos(2 * M_PI * (y - dy / 2.)));
                }
            };
            for (int i = 0; i < N1; ++i)
                for (int j = 0; j < N2; ++j) cc(i, j) = prof(s.x_lb + (i + 0.5) * s.dx, s.y_lb + (j + 0.5) * s.dy);
            Array3d vv;
            vv.resize(N1 + 1 + 2 * g, N2 + 1 + 2 * g, 2, -g, -g);
            for (int i = -g; i <= N1 + g; ++i)
                for (int j = -g; j <= N2 + g; ++j) {
                    vv(i, j, 0) = -L;
                    vv(i, j, 1) = H;
                }
            E.put_c(cc);
            E.put_v(vv);
            double dtmax = s.cfl * std::min(s.dx / L, s.dy / H), t = s.tstart, dt = dtmax;
            std::vector<double> times = s.times;
            if (std::find(times.begin(), times.end(), s.tfinal) == times.end()) times.push_back(s.tfinal);
            std::sort(times.begin(), times.end());
            size_t tidx = 0;
            int pfs = 1;
            double of = 0;
            while (t < s.tfinal) {
                if (tidx < times.size() && t + dt >= times[tidx]) dt = times[tidx++] - t;
                else dt = dtmax;
                E.check(impec_hyperbolic_solve(E.ctx(), E.c, E.u, E.v, dt, &pfs, &of), "impec_hyperbolic_solve");
                t += dt;
            }
            E.get_c(cc);
            double e = 0;
            for (int i = 0; i < N1; ++i)
                for (int j = 0; j < N2; ++j) {
                    double ex = prof(s.x_lb + (i + 0.5) * s.dx, s.y_lb + (j + 0.5) * s.dy);
                    e += s.hyp_norm == L2 ? (ex - cc(i, j)) * (ex - cc(i, j)) : std::fabs(ex - cc(i, j));
                }
            double nrm = s.hyp_norm == L2 ? std::sqrt(s.dx * s.dy * e) : e * s.dx * s.dy;
            std::cout << "\t\tL" << (s.hyp_norm == L2 ? 2 : 1) << ":\t" << nrm << std::endl;
            norm << std::log(s.dx) << "\t" << std::log(nrm) << "\n";
        }
    }
    return true;
}

// ---------------------------------------------------------------- C ABI over the host layer
extern "C" {

impec_status impec_cfg_load(const char* path, impec_params* P, double* tstart, double* tfinal) {
    if (!path || !P) return IMPEC_ERR_ARG;
    try {
        SimParams sp{std::string(path)};
        *P = sp.engine();
        if (tstart) *tstart = sp.tstart;
        if (tfinal) *tfinal = sp.tfinal;
        return IMPEC_OK;
    } catch (const std::exception& e) {
        fprintf(stderr, "%s\n", e.what());
        impec::set_error(e.what());
        return IMPEC_ERR_CONFIG;
    }
}

impec_status impec_cfg_source(const char* path, double* q_host) {
    if (!path || !q_host) return IMPEC_ERR_ARG;
    try {
        SimParams sp{std::string(path)};
        InitializeSourceTerm(sp, q_host, sp.tstart);
        return IMPEC_OK;
    } catch (const std::exception& e) {
        fprintf(stderr, "%s\n", e.what());
        impec::set_error(e.what());
        return IMPEC_ERR_CONFIG;
    }
}

impec_status impec_run_cfg(const char* path, int quiet) {
    if (!path) return IMPEC_ERR_ARG;
    try {
        Impec2DSolver s{std::string(path)};
        if (quiet && !s.sp->is_test) return s.Solve(true) ? IMPEC_OK : IMPEC_ERR_NOT_CONVERGED;
        return s.Run() ? IMPEC_OK : IMPEC_ERR_NOT_CONVERGED;
    } catch (const ConfigError& e) {
        fprintf(stderr, "%s\n", e.what());
        impec::set_error(e.what());
        return IMPEC_ERR_CONFIG;
    } catch (const EngineError& e) {
        fprintf(stderr, "%s\n", e.what());
        impec::set_error(e.what());
        return e.status;
    } catch (const std::exception& e) {
        fprintf(stderr, "%s\n", e.what());
        impec::set_error(e.what());
        return IMPEC_ERR_ARG;
    }
}

}  // extern "C"
