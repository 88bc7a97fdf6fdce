// libconfig-subset parser and SimParams (src/SimParams.cpp:45-468): the same required keys and
// the same validation, reported by ConfigError / IMPEC_ERR_CONFIG instead of exit(1).
#include "SimParams.h"

#include <cctype>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

// ---------------------------------------------------------------- tree lookup
const CfgNode* CfgNode::get(const std::string& name) const {
    for (auto& c : children)
        if (c.first == name) return c.second.get();
    return nullptr;
}
bool CfgNode::lookup(const std::string& name, int& out) const {
    const CfgNode* n = get(name);
    if (!n) return false;
    if (n->kind == INT) { out = (int)n->i; return true; }
    if (n->kind == FLOAT) { out = (int)n->f; return true; }
    return false;
}
bool CfgNode::lookup(const std::string& name, double& out) const {
    const CfgNode* n = get(name);
    if (!n) return false;
    if (n->kind == FLOAT) { out = n->f; return true; }
    if (n->kind == INT) { out = (double)n->i; return true; }
    return false;
}
bool CfgNode::lookup(const std::string& name, bool& out) const {
    const CfgNode* n = get(name);
    if (!n || n->kind != BOOL) return false;
    out = n->b;
    return true;
}
bool CfgNode::lookup(const std::string& name, std::string& out) const {
    const CfgNode* n = get(name);
    if (!n || n->kind != STRING) return false;
    out = n->s;
    return true;
}

// ---------------------------------------------------------------- parser
namespace {
struct Parser {
    const std::string& t;
    std::string fname;
    size_t k = 0;
    int line = 1;
    [[noreturn]] void fail(const std::string& msg) {
        throw ConfigError("Parse error at " + fname + ":" + std::to_string(line) + " - " + msg);
    }
    void skip() {
        for (;;) {
            while (k < t.size() && isspace((unsigned char)t[k])) {
                if (t[k] == '\n') ++line;
                ++k;
            }
            if (k >= t.size()) return;
            if (t[k] == '#' || (t[k] == '/' && k + 1 < t.size() && t[k + 1] == '/')) {
                while (k < t.size() && t[k] != '\n') ++k;
                continue;
            }
            if (t[k] == '/' && k + 1 < t.size() && t[k + 1] == '*') {
                size_t e = t.find("*/", k + 2);
                if (e == std::string::npos) fail("unterminated comment");
                for (size_t q = k; q < e; ++q)
                    if (t[q] == '\n') ++line;
                k = e + 2;
                continue;
            }
            return;
        }
    }
    bool peek(char c) {
        skip();
        return k < t.size() && t[k] == c;
    }
    void expect(char c) {
        if (!peek(c)) fail(std::string("expected '") + c + "'");
        ++k;
    }
    std::string name() {
        skip();
        size_t s = k;
        if (k < t.size() && (isalpha((unsigned char)t[k]) || t[k] == '*')) {
            ++k;
            while (k < t.size() && (isalnum((unsigned char)t[k]) || t[k] == '_' || t[k] == '-' || t[k] == '*')) ++k;
        }
        if (s == k) fail("expected a setting name");
        return t.substr(s, k - s);
    }
    std::shared_ptr<CfgNode> value() {
        skip();
        auto n = std::make_shared<CfgNode>();
        if (k >= t.size()) fail("unexpected end of file");
        char c = t[k];
        if (c == '{') {
            ++k;
            n->kind = CfgNode::GROUP;
            settings(*n, '}');
            expect('}');
        } else if (c == '[' || c == '(') {
            char close = c == '[' ? ']' : ')';
            ++k;
            n->kind = CfgNode::LIST;
            while (!peek(close)) {
                n->children.push_back({"", value()});
                if (peek(',')) ++k;
            }
            expect(close);
        } else if (c == '"') {
            n->kind = CfgNode::STRING;
            ++k;
            std::string s;
            while (k < t.size() && t[k] != '"') {
                if (t[k] == '\\' && k + 1 < t.size()) {
                    char e = t[++k];
                    s += e == 'n' ? '\n' : (e == 't' ? '\t' : e);
                } else {
                    s += t[k];
                }
                ++k;
            }
            if (k >= t.size()) fail("unterminated string");
            ++k;
            n->s = s;
            // adjacent string literals concatenate (libconfig)
            while (peek('"')) {
                auto m = value();
                n->s += m->s;
            }
        } else if (isdigit((unsigned char)c) || c == '-' || c == '+' || c == '.') {
            size_t s = k;
            bool flt = false;
            if (t[k] == '-' || t[k] == '+') ++k;
            while (k < t.size() && (isalnum((unsigned char)t[k]) || t[k] == '.' ||
                                    ((t[k] == '-' || t[k] == '+') && (t[k - 1] == 'e' || t[k - 1] == 'E')))) {
                if (t[k] == '.' || t[k] == 'e' || t[k] == 'E') flt = true;
                ++k;
            }
            std::string num = t.substr(s, k - s);
            if (num.size() > 1 && (num.back() == 'L' || num.back() == 'l')) { num.pop_back(); flt = false; }
            char* end = nullptr;
            if (flt) {
                n->kind = CfgNode::FLOAT;
                n->f = strtod(num.c_str(), &end);
            } else {
                n->kind = CfgNode::INT;
                n->i = strtoll(num.c_str(), &end, 0);
            }
            if (!end || *end) fail("bad number '" + num + "'");
        } else {
            std::string w = name();
            std::string lw;
            for (char ch : w) lw += (char)tolower((unsigned char)ch);
            if (lw == "true" || lw == "false") {
                n->kind = CfgNode::BOOL;
                n->b = lw == "true";
            } else {
                fail("unexpected token '" + w + "'");
            }
        }
        return n;
    }
    void settings(CfgNode& g, char close) {
        while (true) {
            skip();
            if (k >= t.size() || t[k] == close) return;
            std::string nm = name();
            skip();
            if (k < t.size() && (t[k] == '=' || t[k] == ':')) ++k;
            else fail("expected '=' or ':' after '" + nm + "'");
            g.children.push_back({nm, value()});
            if (peek(';') || peek(',')) ++k;
        }
    }
};
}  // namespace

std::shared_ptr<CfgNode> parse_cfg_text(const std::string& text, const std::string& fname) {
    Parser p{text, fname};
    auto root = std::make_shared<CfgNode>();
    root->kind = CfgNode::GROUP;
    p.settings(*root, '\0');
    p.skip();
    if (p.k < text.size()) p.fail("trailing characters");
    return root;
}

std::shared_ptr<CfgNode> parse_cfg_file(const std::string& path) {
    std::ifstream f(path);
    if (!f) throw ConfigError("I/O error while reading file " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    return parse_cfg_text(ss.str(), path);
}

// ---------------------------------------------------------------- SimParams
SimParams::SimParams(const std::string& configfile) { load(parse_cfg_file(configfile)); }
SimParams::SimParams(const std::string& text, bool) { load(parse_cfg_text(text, "<text>")); }

static const CfgNode& group(const CfgNode& root, const char* a, const char* b) {
    const CfgNode* app = root.get(a);
    const CfgNode* g = app ? app->get(b) : nullptr;
    if (!g || g->kind != CfgNode::GROUP) throw ConfigError(std::string("Could not find section <<") + b + ">>!");
    return *g;
}

void SimParams::load(std::shared_ptr<CfgNode> root) {
    cfg = root;
    const CfgNode& gen = group(*root, "application", "general");
    const CfgNode& ell = group(*root, "application", "elliptic");
    const CfgNode& hyp = group(*root, "application", "hyperbolic");
    std::string sstype, ssync;
    // required keys of the <<general>> section (src/SimParams.cpp:57-76)
    if (!(gen.lookup("x_cells", N1) && gen.lookup("y_cells", N2) && gen.lookup("num_ghostcells", p_bounds) &&
          gen.lookup("num_ghostcells", c_bounds) && gen.lookup("x_lb", x_lb) && gen.lookup("x_ub", x_ub) &&
          gen.lookup("y_ub", y_ub) && gen.lookup("y_lb", y_lb) && gen.lookup("starttime", tstart) &&
          gen.lookup("endtime", tfinal) && gen.lookup("I", I) && gen.lookup("log_to_file", log_to_file) &&
          gen.lookup("results_dir", results_dir) && gen.lookup("check_mass_conservation", check_mass_conservation) &&
          gen.lookup("check_noflow_boundary", check_noflow_boundary) && gen.lookup("is_test", is_test) &&
          gen.lookup("source_type", sstype) && gen.lookup("gnuplot", gnuplot) &&
          gen.lookup("check_divergence", check_divergence) && gen.lookup("levelset", levelset) &&
          gen.lookup("syncmode", ssync)))
        throw ConfigError("Could not find one or more items in section <<general>>!");
    if (ssync == "sync") sm = SYNC;
    else if (ssync == "async") sm = ASYNC;
    else throw ConfigError("Config::Synchronization: protocoll is not implemented!");
    if (check_mass_conservation && !gen.lookup("max_mass_frac_error", max_mass_frac_error))
        throw ConfigError("Could not find one or more options in section <<general>>! You need to specify <<max_mass_frac_error>>");
    if (log_to_file && !(gen.lookup("log_skip_steps", log_skip_steps) && gen.lookup("time_matching", time_matching) &&
                         gen.lookup("log_mass_conservation", log_mass_conservation) && gen.lookup("log_dir", log_dir)))
        throw ConfigError("Could not find one or more logging-options in section <<general>>!");
    if (!log_to_file) { log_skip_steps = 0; time_matching = false; }
    if (sstype == "parallel") stype = PARALLEL;
    else if (sstype == "diagonal") stype = DIAGONAL;
    else if (sstype == "horizontal") stype = HORIZONTAL;
    else throw ConfigError("Config::General: source type is not valid!");
    // <<elliptic>> (src/SimParams.cpp:131-180)
    std::string smethod, sbtype, savgproc;
    if (!(ell.lookup("ell_method", smethod) && ell.lookup("bound_type", sbtype) && ell.lookup("eps", eps) &&
          ell.lookup("mu_res", mu_res) && ell.lookup("mu_inj", mu_inj) && ell.lookup("const_bound_val", b_val) &&
          ell.lookup("average_procedure", savgproc)))
        throw ConfigError("Could not find one or more items in <<elliptic>> section!");
    if (sbtype == "neumann") btype = NEUMANN;
    else throw ConfigError("Config::Elliptic: Boundary type is not supported at the moment!");
    if (smethod == "direct") mtype = DIRECT;
    else if (smethod == "cg") mtype = CG;
    else if (smethod == "mg") mtype = MG;
    else if (smethod == "cg_cuda") mtype = CG_CUDA;
    else throw ConfigError("Config::Elliptic: Method is unknown!");
    if (savgproc == "harmonic") avgproc = HARMONIC;
    else if (savgproc == "mean_concentration") avgproc = MEANCONC;
    else throw ConfigError("Config::Elliptic: Averaging procedure is unknown!");
    // <<hyperbolic>> (src/SimParams.cpp:182-222)
    std::string shmethod, sdim;
    if (!(hyp.lookup("hyper_method", shmethod) && hyp.lookup("porosity", porosity) && hyp.lookup("cfl", cfl) &&
          hyp.lookup("inj_fluid_conc", inj_fluid_conc) && hyp.lookup("nu", nu) && hyp.lookup("diffusion", diffusion) &&
          hyp.lookup("alpha_l", alpha_l) && hyp.lookup("alpha_t", alpha_t) &&
          hyp.lookup("dt_diff_limiter", dt_diff_limit) && hyp.lookup("dimensional_splitting", sdim)))
        throw ConfigError("Could not find one or more items in <<hyperbolic>> section!");
    if (shmethod == "waf_split") hmtype = WAFSPLIT;
    else if (shmethod == "waf") hmtype = WAF;
    else if (shmethod == "ctu") hmtype = CTU;
    else if (shmethod == "muscl") hmtype = MUSCL;
    else if (shmethod == "upwind_split") hmtype = UPWINDSPLIT;
    else throw ConfigError("Config::Hyperbolic: Method is unknown!");
    if (sdim == "alternating_sweeps") dim_splitting = ALTERNATING;
    else if (sdim == "x_sweep_first") dim_splitting = X_FIRST;
    else if (sdim == "y_sweep_first") dim_splitting = Y_FIRST;
    else if (sdim == "strang") dim_splitting = STRANG;
    else if (sdim == "parallel") dim_splitting = SYMMETRIC_PARALLEL;
    else throw ConfigError("Config::Hyperbolic: Dimenstional Splitting specification is unknown!");
    // output lists (src/SimParams.cpp:236-243)
    counters.clear();
    times.clear();
    if (const CfgNode* l = gen.get("log_counter_list"))
        for (auto& c : l->children) counters.push_back((int)(c.second->kind == CfgNode::INT ? c.second->i : c.second->f));
    else
        throw ConfigError("Could not find setting log_counter_list");
    if (const CfgNode* l = gen.get("log_time_list"))
        for (auto& c : l->children) times.push_back(c.second->kind == CfgNode::FLOAT ? c.second->f : (double)c.second->i);
    else
        throw ConfigError("Could not find setting log_time_list");
    // <<test>> (src/SimParams.cpp:246-317)
    if (is_test) {
        const CfgNode& ts = group(*root, "application", "test");
        std::string comp, sprofile;
        int ihypnorm = 1;
        ts.lookup("component", comp);
        ts.lookup("testno", testno);
        ts.lookup("num_result_file", num_result_file);
        ts.lookup("ex_result_file", ex_result_file);
        ts.lookup("norm_file", norm_file);
        ts.lookup("initial_x_cells", init_x_cells);
        ts.lookup("initial_y_cells", init_y_cells);
        ts.lookup("num_u_file", num_u_file);
        ts.lookup("ex_u_file", ex_u_file);
        ts.lookup("num_v_file", num_v_file);
        ts.lookup("ex_v_file", ex_v_file);
        ts.lookup("levels", levels);
        ts.lookup("profile", sprofile);
        ts.lookup("hyp_norm", ihypnorm);
        if (comp == "elliptic") test_component = ELLIPTIC;
        else if (comp == "hyperbolic") test_component = HYPERBOLIC;
        else throw ConfigError("TestComponent> Config::General: source type is not valid!");
        if (sprofile == "sine") hyp_test = SINE;
        else if (sprofile == "tophat") hyp_test = TOPHAT;
        else if (sprofile == "gaussbell") hyp_test = GAUSS;
        else if (sprofile == "horizontal_sine") hyp_test = HSINE;
        else throw ConfigError("TestComponent> Config:: Test profile is not valid!");
        if (ihypnorm == 1) hyp_norm = L1;
        else if (ihypnorm == 2) hyp_norm = L2;
        else throw ConfigError("TestComponent> Config:: Norm is not supported!");
    }
    if (!gen.lookup("init_file", init_file)) init_file = "";
    std::string sti;
    if (!(hyp.lookup("time_integration", sti) && hyp.lookup("ti_eps", ti_eps)))
        throw ConfigError("Could not find property <<time_integration>> or <<ti_eps>>!");
    ti = TR;  // src/SimParams.cpp:335
    // <<wells>> (src/SimParams.cpp:357-404)
    const CfgNode& wl = group(*root, "application", "wells");
    std::string swp, smode;
    if (!(wl.lookup("well_profile", swp) && wl.lookup("well_rc", well_rc) && wl.lookup("q_freq", q_freq) &&
          wl.lookup("q_rand_max", q_rand_max) && wl.lookup("front_const_width", front_const_width) &&
          wl.lookup("well_width", well_width) && wl.lookup("front_rand_width", front_rand_width) &&
          wl.lookup("q_high_multiple", q_high_multiple) && wl.lookup("mode", smode)))
        throw ConfigError("Could not find one or more items in section <<wells>>!");
    if (smode == "pulsing") im = PULSING;
    else if (smode == "linear") im = LINEAR;
    else if (smode == "constant") im = CONSTANT;
    else throw ConfigError("Unknown injection mode: " + smode);
    if (swp == "circle") well_profile = CIRCULAR;
    else if (swp == "gauss") well_profile = GAUSSIAN;
    else if (swp == "one_cell") well_profile = ONECELL;
    else throw ConfigError("Unknown profile <<wells>>!");
    // <<parabolic>> (src/SimParams.cpp:406-428)
    const CfgNode& pa = group(*root, "application", "parabolic");
    std::string spm;
    if (!(pa.lookup("para_method", spm) && pa.lookup("eps", para_eps)))
        throw ConfigError("Could not find one or more items in section <<parabolic>>!");
    if (spm == "crank-nicolson") ptype = CRANKNICOLSON;
    else if (spm == "explicit") ptype = EXPLICIT;
    else throw ConfigError("Unknown parabolic solver <<" + spm + ">>!");
    if (ptype == CRANKNICOLSON && mtype != MG)
        throw ConfigError("SimParams::InvalidOptions> The Crank-Nicolson scheme requires a Multigrid-Solver. Change ell_method to MG!");
    // engine options: optional group application.gb300 (unknown to the reference, ignored by it)
    const CfgNode* app = root->get("application");
    if (const CfgNode* e = app ? app->get("gb300") : nullptr) {
        std::string prec;
        if (e->lookup("precision", prec)) {
            if (prec == "fp64") precision = IMPEC_PREC_FP64;
            else if (prec == "mixed") precision = IMPEC_PREC_MIXED;
            else throw ConfigError("gb300.precision must be \"fp64\" or \"mixed\"");
        }
        e->lookup("molecular_diffusion", Dm);
        e->lookup("max_cycles", max_cycles);
        bool b;
        if (e->lookup("warm_start", b)) warm_start = b;
        if (e->lookup("peaceman_guard", b)) peaceman_guard = b;
        if (e->lookup("cfl_porosity", b)) cfl_porosity = b;
        if (e->lookup("learned_weights", learned_weights) && !learned_weights.empty())
            warm_start = 1;  // the network moves the previous pressure
        if (e->lookup("learned_factor", learned_factor) &&
            !(learned_factor == 1 || learned_factor == 2 || learned_factor == 4 || learned_factor == 8 ||
              learned_factor == 16))
            throw ConfigError("gb300.learned_factor must be 1, 2, 4, 8 or 16");
    }
    v_bounds = p_bounds;  // src/SimParams.cpp:448
    dx = (x_ub - x_lb) / N1;
    dy = (y_ub - y_lb) / N2;
    M = N1 * N2;
    sigma0 *= dx;
    sigma1 *= dx;
    sigma2 *= dx;
    if (stype == PARALLEL && (dx != dy || N1 != N2))
        throw ConfigError("ERROR: This resolution is not supported for the parallel configuration. The module "
                          "ParallelProjector assumes square grid blocks and equal resolution in both dimensions.");
    if (N1 < 2 || N2 < 2) throw ConfigError("x_cells and y_cells must be at least 2");
    if (p_bounds < 2) throw ConfigError("num_ghostcells must be at least 2 (MUSCL needs two ghost layers)");
}

impec_params SimParams::engine() const {
    impec_params P;
    impec_default_params(&P, N1, N2);
    P.x_lb = x_lb; P.x_ub = x_ub; P.y_lb = y_lb; P.y_ub = y_ub;
    P.mu_res = mu_res; P.mu_inj = mu_inj;
    P.avgproc = avgproc == HARMONIC ? IMPEC_HARMONIC : IMPEC_MEANCONC;
    P.nu = nu;
    P.porosity = porosity; P.cfl = cfl; P.inj_fluid_conc = inj_fluid_conc; P.I = I;
    P.diffusion = diffusion; P.alpha_l = alpha_l; P.alpha_t = alpha_t; P.Dm = Dm;
    P.ptype = ptype == CRANKNICOLSON ? IMPEC_CRANKNICOLSON : IMPEC_EXPLICIT;
    P.dt_diff_limit = dt_diff_limit;
    P.dim_splitting = (int)dim_splitting;
    P.hmtype = hmtype == UPWINDSPLIT ? IMPEC_UPWINDSPLIT
               : hmtype == WAFSPLIT  ? IMPEC_WAFSPLIT
               : hmtype == WAF       ? IMPEC_WAF
               : hmtype == CTU       ? IMPEC_CTU
                                     : IMPEC_MUSCL;
    P.stype = stype == PARALLEL ? IMPEC_PARALLEL : (stype == DIAGONAL ? IMPEC_DIAGONAL : IMPEC_HORIZONTAL);
    P.is_test = is_test; P.testno = testno;
    P.bc = is_test ? IMPEC_BC_PERIODIC : IMPEC_BC_NEUMANN;
    P.eps = eps; P.para_eps = para_eps;
    P.peaceman_guard = peaceman_guard; P.cfl_porosity = cfl_porosity; P.precision = precision;
    P.max_cycles = max_cycles; P.warm_start = warm_start;
    return P;
}
