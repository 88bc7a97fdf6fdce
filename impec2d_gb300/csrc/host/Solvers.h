// The reference's solver class surface (pw359/Impec2D src/*.h), backed by the GB300 engine.
//
// Names and roles follow the reference: Impec2DSolver (src/Impec2DSolver.h:40-80),
// EllipticSolver / MGSolver (src/EllipticSolver.h:15-110, src/MGSolver.h), HyperbolicSolver /
// HyperbolicSplitSolver / MUSCLSplitSolver / UpwindSplitSolver (src/HyperbolicSolver.h:15-42,
// src/HyperbolicSplitSolver.h, src/MUSCLSplitSolver.h, src/UpwindSplitSolver.h), and
// TimeIntegrator / TRIntegrator (src/TimeIntegrator.h, src/TRIntegrator.h).  Host arrays keep
// the reference's ghost-indexed layouts; each call copies them to the device context and back.
// Errors are reported by return value or EngineError, never by exit().
#pragma once
#include <stdexcept>
#include <string>
#include <vector>

#include "Arrays.h"
#include "SimParams.h"
#include "impec2d.h"

struct EngineError : std::runtime_error {
    impec_status status;
    EngineError(impec_status s, const std::string& what) : std::runtime_error(what), status(s) {}
};

// Shared device context of one grid (owned by whoever creates the solvers).
class Engine {
public:
    explicit Engine(const SimParams& sp);
    ~Engine();
    Engine(const Engine&) = delete;
    Engine& operator=(const Engine&) = delete;
    impec_ctx* ctx() const { return ctx_; }
    double *c, *p, *u, *v, *q;  // device state
    void check(impec_status s, const char* what) const;
    // host (reference layout, ghost width g) <-> device state
    void put_c(const Array2d& c_host);
    void get_c(Array2d& c_host);
    void get_p(Array2d& p_host);
    void put_v(const Array3d& v_host);
    void get_v(Array3d& v_host);
    void put_q(const double* q_host);
    // Impec2DSolver::Project on the device: c (field 0) or p (field 1) of a parallel run onto the
    // dN1 x dN2 diagonal grid, into `a` with a zero ghost ring of `bounds`
    void project_diagonal(int field, int dN1, int dN2, Array2d& a, int bounds);
    int N1, N2, g;

private:
    void attach_learned(const SimParams& sp);
    impec_ctx* ctx_ = nullptr;
    impec_net* net_ = nullptr;  // learned warm start (gb300.learned_weights), or none
};

class EllipticSolver {
protected:
    SimParams* sp;
    Engine* eng;
    int last_its = 0, last_parabolic_its = 0, total_its = 0, calls = 0;
    double nu;

public:
    EllipticSolver(SimParams* sp, Engine* eng);
    virtual ~EllipticSolver() = default;
    virtual bool SolveLinearMultigrid(Array2d& c_c, int c_bounds, Array2d& p_c, int p_bounds, const double* q_v) = 0;
    bool Solve(Array2d& p, Array2d& c, double* q);
    void CalcVelocities(Array2d& p, Array3d& v, Array2d& c);
    void SetNu(double nu);
    int GetLastIts() const { return last_its; }
    int GetLastParabolicIts() const { return last_parabolic_its; }
    double GetAvgIts() const { return calls > 0 ? (double)total_its / calls : 0.0; }
    double last_relres = 0;
};

class MGSolver : public EllipticSolver {
public:
    MGSolver(SimParams* sp, Engine* eng) : EllipticSolver(sp, eng) {}
    bool SolveLinearMultigrid(Array2d& c_c, int c_bounds, Array2d& p_c, int p_bounds, const double* q_v) override;
    bool Solve_Parabolic_cc_to_c(Array2d& c_c, int c_bounds, const Array3d& v, int v_bounds, double dt);
};

class TimeIntegrator {
protected:
    SimParams* sp;
    Engine* eng;
    double total_mass_outflux = 0;

public:
    TimeIntegrator(SimParams* sp, Engine* eng) : sp(sp), eng(eng) {}
    virtual ~TimeIntegrator() = default;
    double GetTotalMassOutflux() const { return total_mass_outflux; }
    virtual int Integrate(Array2d& c, const double* q, double dt) = 0;
    int IntegrateSubcycle(Array2d& c, const double* q, double dt) { return Integrate(c, q, dt); }
};

class TRIntegrator : public TimeIntegrator {
public:
    using TimeIntegrator::TimeIntegrator;
    int Integrate(Array2d& c, const double* q, double dt) override;
};

enum SWEEP { X_SWEEP, Y_SWEEP };

class HyperbolicSolver {
protected:
    SimParams* sp;
    Engine* eng;
    MGSolver* mg = nullptr;
    TRIntegrator ti;
    double total_mass_outflux = 0;
    SWEEP prev_first_sweep = Y_SWEEP;
    bool SourceSplit(Array2d& c, const double* q, double dt);

public:
    HyperbolicSolver(SimParams* sp, Engine* eng) : sp(sp), eng(eng), ti(sp, eng) {}
    virtual ~HyperbolicSolver() = default;
    virtual bool Solve(Array2d& c, const Array3d& v, const double* q, double dt) = 0;
    double GetTotalMassOutflux() const { return total_mass_outflux; }
    void FillBoundaries(Array2d& c);
    double MaxStableTimestep(const Array2d& c, const Array3d& v);
    bool DiffusionSplit(Array2d& c, const Array3d& v, double dt);
    void AssignMGSolver(MGSolver* m) { mg = m; }
};

class HyperbolicSplitSolver : public HyperbolicSolver {
protected:
    bool AdvectSplit(Array2d& c, const Array3d& v, const double* q, double dt);

public:
    using HyperbolicSolver::HyperbolicSolver;
    bool Solve(Array2d& c, const Array3d& v, const double* q, double dt) override;
    bool Advect_X(Array2d& c, const Array3d& v, double dt);
    bool Advect_Y(Array2d& c, const Array3d& v, double dt);
};

// The scheme is the engine's hmtype; these classes exist so that code naming them keeps working.
class MUSCLSplitSolver : public HyperbolicSplitSolver {
public:
    using HyperbolicSplitSolver::HyperbolicSplitSolver;
};
class UpwindSplitSolver : public HyperbolicSplitSolver {
public:
    using HyperbolicSplitSolver::HyperbolicSplitSolver;
};

struct DiagState {  // src/Impec2DSolver.h:16-25
    int ctr;
    int its;
    double t, dt, mass_err, diff_err, vel_err, fillperdt;
};

class Impec2DSolver {
    Array2d p, c;
    Array3d v;
    std::vector<double> q;
    Engine* eng = nullptr;
    EllipticSolver* es = nullptr;
    HyperbolicSolver* hs = nullptr;
    int myid, num_procs;

public:
    SimParams* sp;
    Impec2DSolver(const std::string& configfile, int myid = 0, int num_procs = 1);
    virtual ~Impec2DSolver();
    bool Run();
    // resident-state time loop; quiet suppresses the per-step console line
    bool Solve(bool quiet = false);
    const Array2d& concentration() const { return c; }
    const Array2d& pressure() const { return p; }
    const Array3d& velocity() const { return v; }
    std::vector<DiagState> diag;

private:
    void Initialize();
    void ResizeArrays();
    void InitializeConcentration();
    void InitializeSource();
    void WriteDiagnostics(const std::vector<DiagState>& ds);
    void LogResults(const std::string& postfix);
    double CalculateMassError(double t, double mass);
    bool TestComponent();
};

// Printer (src/Printer.cpp:98-188): "x y value" dumps, blank line after each i.
void PrintDToPlotFile(const std::string& filename, const Array2d& a, double x_lb, double y_lb, double dx, double dy,
                      int skip_bounds);
void PrintVelToPlotFile(const std::string& ufile, const std::string& vfile, const Array3d& a, double x_lb, double y_lb,
                        double dx, double dy, int skip_bounds);
// Source term of InitializeSource (src/Impec2DSolver.cpp:241-280 and src/Util.cpp:444-639).
void InitializeSourceTerm(const SimParams& sp, double* q, double t);
