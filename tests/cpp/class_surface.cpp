// Drives the engine's C++ class surface -- the reference's class names and signatures
// (src/EllipticSolver.h:61-69, src/HyperbolicSolver.h:27-39, src/HyperbolicSplitSolver.h,
// src/TimeIntegrator.h, src/MGSolver.h) -- on reference-layout host arrays, the way code written
// against the reference calls it.  Test infrastructure: tests/test_gpu_class_surface.py builds
// it against libimpec2d.so, feeds it the inputs of a reference fixture and compares what it
// writes with the reference's own outputs.
//
//   class_surface <case.cfg> <dir> <dt>
// reads <dir>/{c,v,v_of_p,p,q}.bin (raw doubles, reference layouts with ghosts) and writes
// <dir>/out_{p_solve,v_of_p,tr_c,advect_x,advect_y,advect_split,cn_c,hyp_c}.bin and out_scalars.txt.
#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "Solvers.h"

namespace {

std::vector<double> load(const std::string& path, size_t n) {
    std::vector<double> v(n);
    std::ifstream f(path, std::ios::binary);
    if (!f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(n * sizeof(double))))
        throw std::runtime_error("cannot read " + path);
    return v;
}
void save(const std::string& path, const double* a, size_t n) {
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(a), (std::streamsize)(n * sizeof(double)));
}

// A subclass only to reach the split driver's protected AdvectSplit, as a reference subclass can.
class SplitProbe : public MUSCLSplitSolver {
public:
    using MUSCLSplitSolver::MUSCLSplitSolver;
    bool Split(Array2d& c, const Array3d& v, double dt) { return AdvectSplit(c, v, nullptr, dt); }
};

}  // namespace

int main(int argc, char** argv) {
    if (argc != 4) {
        std::cerr << "usage: class_surface <case.cfg> <dir> <dt>\n";
        return 2;
    }
    try {
        SimParams sp(argv[1]);
        const std::string dir = argv[2];
        const double dt = std::stod(argv[3]);
        const int g = sp.c_bounds, N1 = sp.N1, N2 = sp.N2;
        const size_t ns = (size_t)(N1 + 2 * g) * (N2 + 2 * g), nv = (size_t)(N1 + 1 + 2 * g) * (N2 + 1 + 2 * g) * 2;
        Engine eng(sp);
        MGSolver mg(&sp, &eng);
        SplitProbe hs(&sp, &eng);
        hs.AssignMGSolver(&mg);
        TRIntegrator tr(&sp, &eng);

        auto scalar = [&](const std::string& name) {
            Array2d a(N1 + 2 * g, N2 + 2 * g, -g, -g);
            std::vector<double> h = load(dir + "/" + name + ".bin", ns);
            std::copy(h.begin(), h.end(), a.data());
            return a;
        };
        auto vel = [&](const std::string& name) {
            Array3d a;
            a.resize(N1 + 1 + 2 * g, N2 + 1 + 2 * g, 2, -g, -g);
            std::vector<double> h = load(dir + "/" + name + ".bin", nv);
            std::copy(h.begin(), h.end(), a.data());
            return a;
        };
        std::vector<double> q = load(dir + "/q.bin", (size_t)N1 * N2);
        std::ofstream sc(dir + "/out_scalars.txt");
        sc.precision(17);

        // EllipticSolver::Solve -> MGSolver::SolveLinearMultigrid
        Array2d c = scalar("c"), p(N1 + 2 * g, N2 + 2 * g, -g, -g);
        const bool ok = mg.Solve(p, c, q.data());
        save(dir + "/out_p_solve.bin", p.data(), ns);
        sc << "solve_ok " << ok << "\nits " << mg.GetLastIts() << "\nrelres " << mg.last_relres << "\n";
        // EllipticSolver::CalcVelocities on the reference's pressure
        Array2d pr = scalar("p");
        Array3d v(vel("v"));
        v = 0.0;
        mg.CalcVelocities(pr, v, c);
        save(dir + "/out_v_of_p.bin", v.data(), nv);
        // HyperbolicSolver::MaxStableTimestep
        Array3d vp = vel("v_of_p");
        sc << "dt " << hs.MaxStableTimestep(c, vp) << "\n";
        // TRIntegrator::Integrate
        Array2d ct = scalar("c");
        tr.Integrate(ct, q.data(), dt);
        save(dir + "/out_tr_c.bin", ct.data(), ns);
        sc << "tr_outflux " << tr.GetTotalMassOutflux() << "\n";
        // HyperbolicSplitSolver::Advect_X / Advect_Y with the fixture's random velocities
        Array3d vr = vel("v");
        Array2d cx = scalar("c");
        hs.Advect_X(cx, vr, dt);
        save(dir + "/out_advect_x.bin", cx.data(), ns);
        Array2d cy = scalar("c");
        hs.Advect_Y(cy, vr, dt);
        save(dir + "/out_advect_y.bin", cy.data(), ns);
        // AdvectSplit (the cfg's splitting) with the velocities of the reference's pressure
        Array2d cs = scalar("c");
        hs.Split(cs, vp, dt);
        save(dir + "/out_advect_split.bin", cs.data(), ns);
        // MGSolver::Solve_Parabolic_cc_to_c (one CN half step)
        Array2d cc = scalar("c");
        const bool cn_ok = mg.Solve_Parabolic_cc_to_c(cc, g, vp, g, 0.5 * dt);
        save(dir + "/out_cn_c.bin", cc.data(), ns);
        sc << "cn_ok " << cn_ok << "\n";
        // HyperbolicSplitSolver::Solve (source, CN, advection, source, CN)
        SplitProbe hs2(&sp, &eng);
        hs2.AssignMGSolver(&mg);
        Array2d ch = scalar("c");
        const bool h_ok = hs2.Solve(ch, vp, q.data(), dt);
        save(dir + "/out_hyp_c.bin", ch.data(), ns);
        sc << "hyp_ok " << h_ok << "\nhyp_outflux " << hs2.GetTotalMassOutflux() << "\n";
    } catch (const std::exception& e) {
        std::cerr << "class_surface: " << e.what() << "\n";
        return 1;
    }
    return 0;
}
