// Run parameters read from a libconfig-format .cfg file.  Field names and meanings follow the
// reference's SimParams (src/SimParams.h:29-164) so that existing configuration files and code
// that reads these fields carry over.  Parsing errors throw ConfigError instead of exiting.
#pragma once
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "impec2d.h"

enum M_Type { DIRECT, CG, CG_CUDA, MG };
enum HM_Type { UPWINDSPLIT, WAFSPLIT, WAF, CTU, MUSCL };
enum S_Type { PARALLEL, DIAGONAL, HORIZONTAL };
enum Solver_Test { ELLIPTIC, HYPERBOLIC };
enum Hyp_Test { SINE, TOPHAT, GAUSS, HSINE };
enum Hyp_Norm { L1, L2 };
enum B_Type { DIRICHLET, SHIFTEDNEUMANN, NEUMANN };
enum DIM_SPLITTING { ALTERNATING, X_FIRST, Y_FIRST, STRANG, SYMMETRIC_PARALLEL };
enum AVG_PROC { MEANCONC, HARMONIC };
enum TIME_INTEGRATOR { TR, HEUN, FE, HEUNFE };
enum WELL { CIRCULAR, GAUSSIAN, ONECELL };
enum P_Type { EXPLICIT, CRANKNICOLSON };
enum SYNCMODE { SYNC, ASYNC };
enum INJ_MODE { PULSING, LINEAR, CONSTANT };

struct ConfigError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// Parsed libconfig value tree (the subset the examples use: groups, scalars, strings, lists).
struct CfgNode {
    enum Kind { GROUP, LIST, INT, FLOAT, BOOL, STRING } kind = GROUP;
    long long i = 0;
    double f = 0;
    bool b = false;
    std::string s;
    std::vector<std::pair<std::string, std::shared_ptr<CfgNode>>> children;  // group / list items
    const CfgNode* get(const std::string& name) const;
    bool lookup(const std::string& name, int& out) const;
    bool lookup(const std::string& name, double& out) const;
    bool lookup(const std::string& name, bool& out) const;
    bool lookup(const std::string& name, std::string& out) const;
};
std::shared_ptr<CfgNode> parse_cfg_text(const std::string& text, const std::string& fname);
std::shared_ptr<CfgNode> parse_cfg_file(const std::string& path);

class SimParams {
public:
    std::shared_ptr<CfgNode> cfg;
    double tfinal, tstart;
    int c_bounds, p_bounds, v_bounds;
    int N1, N2, M;
    double x_lb, y_lb, x_ub, y_ub;
    double dx, dy;
    M_Type mtype;
    P_Type ptype;
    HM_Type hmtype;
    S_Type stype;
    double I, porosity;
    bool log_to_file, time_matching;
    int log_skip_steps;
    std::string log_dir;
    bool log_delete_content_first = false;
    std::string results_dir;
    std::vector<int> counters;
    std::vector<double> times;
    bool log_mass_conservation = false, check_mass_conservation, check_noflow_boundary;
    double max_mass_frac_error = 0;
    double inj_fluid_conc, cfl, b_val;
    B_Type btype;
    double eps, para_eps, mu_res, mu_inj;
    Solver_Test test_component = ELLIPTIC;
    int testno = 1;
    std::string num_result_file, ex_result_file, norm_file, ex_u_file, num_u_file, ex_v_file, num_v_file;
    int levels = 1, init_x_cells = 0, init_y_cells = 0;
    bool is_test;
    Hyp_Test hyp_test = SINE;
    Hyp_Norm hyp_norm = L1;
    bool gnuplot;
    DIM_SPLITTING dim_splitting;
    bool check_divergence;
    AVG_PROC avgproc;
    std::string init_file;
    TIME_INTEGRATOR ti;
    double ti_eps;
    double nu;
    bool diffusion;
    double alpha_l, alpha_t;
    bool levelset;
    int ls_bounds = 3, ls_flag_neigh = 4;
    bool ls_flagged_diff = false;
    int ls_iter = 10;
    double well_rc;
    WELL well_profile;
    double q_freq, q_rand_max;
    int front_const_width, front_rand_width;
    double q_high_multiple;
    INJ_MODE im;
    double well_width;
    double dt_diff_limit;
    bool ls_mod_diff = false;
    double sigma1 = 0, sigma2 = 0, sigma0 = 0;
    SYNCMODE sm;
    // engine options (optional group application.gb300; absent = reference behaviour)
    double Dm = 0.0;
    int precision = IMPEC_PREC_FP64, max_cycles = 100, warm_start = 0, peaceman_guard = 1, cfl_porosity = 0;
    // learned warm start: trained parameters (.npy of float32, impec_net_parameters order) and
    // the feature averaging factor (0: N1 / 256 rounded down to 1, 2, 4, 8 or 16)
    std::string learned_weights;
    int learned_factor = 0;

    explicit SimParams(const std::string& configfile);
    SimParams(const std::string& text, bool from_text);
    virtual ~SimParams() = default;
    // Engine parameters for the grid currently described by N1, N2, dx, dy.
    impec_params engine() const;

private:
    void load(std::shared_ptr<CfgNode> root);
};
