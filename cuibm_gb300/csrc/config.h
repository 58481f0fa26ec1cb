// Case description of one simulation: the reference's parameterDB sections
// ("inputs", "flow", "simulation", "velocitySolve", "PoissonSolve") as a typed
// struct, plus the grid and body descriptions from domain.yaml/bodies.yaml.
#pragma once
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace cuibm {

enum Boundary { XMINUS = 0, XPLUS = 1, YMINUS = 2, YPLUS = 3 };
enum BcType { DIRICHLET = 0, NEUMANN, CONVECTIVE, PERIODIC, SPECIAL };
enum Precond { PC_NONE = 0, PC_DIAGONAL = 1, PC_SMOOTHED_AGGREGATION = 2, PC_AINV = 3 };
enum Krylov { KRYLOV_BICGSTAB = 0, KRYLOV_CG = 1 };
enum Precision { PRECISION_FP64 = 0, PRECISION_MIXED = 1 };
enum SolverType { ST_NAVIERSTOKES = 0, ST_FADLUN = 1, ST_OSC = 2, ST_FSI = 3, ST_LUO = 4 };

struct LinearSolve {
    std::string solver = "CG";   // parsed; see Params::krylov_* for what runs
    int precond = PC_DIAGONAL;
    double tolerance = 1e-5;
    int maxIterations = 10000;
    int precision = PRECISION_FP64;  // `precision: MIXED`: FP32 multigrid cycles / inner solves, FP64 Krylov
    // `strengthThreshold`: smoothed aggregation links i and j when |a_ij| >= theta sqrt(|a_ii a_jj|)
    // (either way round).  0 (CUSP's default) makes every entry strong.  On the stretched cylinder
    // grids theta = 0.05 halves the Poisson iterations (anisotropic cells coarsen along their strong
    // direction) at about twice the hierarchy's operator complexity.  Unset (-1): 0, except 0.05
    // for the embedded method with a moving body, where theta = 0 broke down (krylov.cu)
    double strength = -1.0;
};

struct AxisDesc {
    double start = 0, mid_h = 0;
    std::vector<double> ends, ratios;
};

struct BodyDesc {
    std::string type;
    // circle
    double cx = 0, cy = 0, R = 0, mid_h = 0;
    int numPoints = 0;
    bool selfSize = false;
    // explicit points (type: points)
    std::vector<double> X, Y;
    // prescribed motion (luo_base/move.cu): x = xC sin(2 pi f t + xPhase), u = uC cos(2 pi f t + uPhase)
    double xCoefficient = 0, yCoefficient = 0, uCoefficient = 0, vCoefficient = 0;
    double xfrequency = 0, yfrequency = 0, xPhase = 0, yPhase = 0, uPhase = 0, vPhase = 0;
};

struct BC {
    int type = DIRICHLET;
    double value = 0;
};

struct Params {
    // inputs
    std::string caseFolder;
    int deviceNumber = 0;
    int solverBlocks = 0;   // -solverBlocks: blocks of the persistent solves (0: one per SM)
    int solverThreads = 0;  // -solverThreads: their block size (0: 512)
    int solverPack = 1;     // -solverPack 2: FP64 persistent solves built for two blocks per SM
                            // (64 registers a thread), so two solves can share an SM
    int saStructured = -1;  // -saStructured 1 / 0: the Poisson system's structured smoothed
                            // aggregation wherever it applies / never (-1: from 200k unknowns)
    // flow
    double nu = 0.01, uInitial = 1.0, vInitial = 0.0, uPerturb = 0.0, vPerturb = 0.0;
    BC bc[4][2];
    // simulation
    double dt = 0.02, scaleCV = 2.0;
    int nt = 100, nsave = 100, startStep = 0, VIV = 0, Ured = 3;
    bool restart = false;
    int solverType = ST_NAVIERSTOKES;
    LinearSolve velocity, poisson;
    // grid and bodies
    AxisDesc axis[2];
    double midH = 0;  // mid_h of the direction listed last in domain.yaml (the reference's domain::mid_h)
    std::vector<BodyDesc> bodies;
    // build-specific keys (absent from reference cases; ignored by the reference)
    int krylovVelocity = KRYLOV_BICGSTAB;
    int krylovPoisson = KRYLOV_BICGSTAB;
    bool writeOutput = true;
};

// Parses caseFolder/{simParams,flow,domain,bodies}.yaml with the reference's
// defaults and the command-line overrides (-nu, -dt, -nt, -nsave, -scaleCV,
// -uPerturb, -vPerturb, -velocityTol, -poissonTol, -caseFolder, -deviceNumber).
// Returns an empty string on success, else the error message.
std::string load_case(const std::string &folder, int argc, const char **argv, Params &P);

}  // namespace cuibm
