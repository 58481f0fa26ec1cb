// Output files in the reference's formats, so its post-processing scripts read
// the library's output unchanged:
//   grid             src/io/io.cu:428-444 (int nx, nx+1 doubles, int ny, ny+1 doubles; the
//                    reference writes one double past the cell centres - here the domain
//                    end coordinate)
//   NNNNNNN/q        src/io/io.cu:459-488 (int N, N doubles of uhat), every nsave steps
//   NNNNNNN/lambda   same, pressure
//   NNNNNNN/bodies   src/bodies.cu:459-471 (body point coordinates)
//   iterations       NavierStokesSolver.cu:350 (timeStep, velocity and Poisson iterations)
//   forces           luoIBM.cu:76-78 (time, Fx, Fy); fadlunModified.cu:64-78 (time, Fx,
//                    FxX, FxY, FxU, Fy)
//   midPosition      luo_base.cu:193-205 (timeStep, X, Y, U, V)
// and one file the reference does not write:
//   NNNNNNN/state    every nsave steps beside q and lambda: what a step reads from the
//                    one before it (velocity with its ghost values, the velocity solve's
//                    start, the convection term for Adams-Bashforth, pressure, the
//                    boundary arrays the convective outflow updates, the body).  With
//                    `restart: true` and `startStep: k` initialise reads k/state and the
//                    run continues as if it had not stopped.  The reference's restart
//                    flag only sets the step counter (parseSimulationFile.cu:99-106)
//                    and starts from the initial condition.
#include <sys/stat.h>

#include <algorithm>
#include <cstdio>
#include <vector>

#include "solver.h"

namespace cuibm {

void write_grid_file(Context &c)
{
    std::string f = c.P.caseFolder + "/grid";
    FILE *fp = fopen(f.c_str(), "wb");
    if (!fp) throw InputError("cannot write " + f);
    auto axis = [&](const Axis &a, double end) {
        int n = a.n;
        std::vector<double> v(a.centre);
        v.push_back(end);
        fwrite(&n, sizeof(int), 1, fp);
        fwrite(v.data(), sizeof(double), v.size(), fp);
    };
    axis(c.gx, c.P.axis[0].ends.back());
    axis(c.gy, c.P.axis[1].ends.back());
    fclose(fp);
}

// io::writeInfoFile (io/io.cu:406-420): the run's summary for the post-processing
// scripts, "--key<TAB>value" with the key right-aligned in 20 columns, numbers as an
// ostream prints them (6 significant digits)
void write_info_file(Context &c)
{
    std::string f = c.P.caseFolder + "/run.info";
    FILE *fp = fopen(f.c_str(), "w");
    if (!fp) throw InputError("cannot write " + f);
    fprintf(fp, "%20s\t%d\n", "--nx", c.g.nx);
    fprintf(fp, "%20s\t%d\n", "--ny", c.g.ny);
    fprintf(fp, "%20s\t%d\n", "--startStep", c.P.startStep);
    fprintf(fp, "%20s\t%d\n", "--nt", c.P.nt);
    fprintf(fp, "%20s\t%d\n", "--nsave", c.P.nsave);
    fprintf(fp, "%20s\t%g\n", "--dt", c.P.dt);
    fprintf(fp, "%20s\t%d\n", "--vortlim", 15);
    fprintf(fp, "%20s\t%s\n", "--folder", c.P.caseFolder.c_str());
    fprintf(fp, "%20s\t%g\n", "--nu", c.P.nu);
    fclose(fp);
}

static void write_array(const std::string &path, const std::vector<double> &v)
{
    FILE *fp = fopen(path.c_str(), "wb");
    if (!fp) throw InputError("cannot write " + path);
    int n = (int)v.size();
    fwrite(&n, sizeof(int), 1, fp);
    fwrite(v.data(), sizeof(double), v.size(), fp);
    fclose(fp);
}

namespace {
const char kStateMagic[8] = {'C', 'U', 'I', 'B', 'M', 'R', 'S', '1'};

// the device arrays of the restart state, in file order
std::vector<std::pair<double *, size_t>> state_arrays(Context &c)
{
    const size_t nUV = c.g.nUV, nP = c.g.nP, bx = 2 * (size_t)c.g.ny - 1, by = 2 * (size_t)c.g.nx - 1;
    std::vector<std::pair<double *, size_t>> S = {{c.u, nUV},          {c.uhat, nUV},        {c.N, nUV},
                                                  {c.p, nP},           {c.bc[XMINUS], bx},   {c.bc[XPLUS], bx},
                                                  {c.bc[YMINUS], by},  {c.bc[YPLUS], by}};
    if (c.has_body) {
        const size_t nb = c.body.total;
        for (double *a : {c.ib.bx, c.ib.by, c.ib.uB, c.ib.vB, c.ib.uBk, c.ib.vBk}) S.push_back({a, nb});
        S.push_back({c.ib.motion, 8});
    }
    return S;
}
}  // namespace

static void write_restart_state(Context &c, const std::string &dir)
{
    auto S = state_arrays(c);
    std::vector<std::vector<double>> host;
    for (auto &a : S) {
        host.emplace_back(a.second);
        CUIBM_TRY(cudaMemcpyAsync(host.back().data(), a.first, a.second * sizeof(double), cudaMemcpyDeviceToHost,
                                  c.stream));
    }
    CUIBM_TRY(cudaStreamSynchronize(c.stream));
    const std::string path = dir + "/state";
    FILE *fp = fopen(path.c_str(), "wb");
    if (!fp) throw InputError("cannot write " + path);
    const int head[6] = {1, c.g.nx, c.g.ny, c.timeStep, c.has_body ? c.body.total : 0, (int)S.size()};
    fwrite(kStateMagic, 1, 8, fp);
    fwrite(head, sizeof(int), 6, fp);
    for (auto &h : host) fwrite(h.data(), sizeof(double), h.size(), fp);
    fclose(fp);
}

void read_restart_state(Context &c)
{
    char path[4096];
    snprintf(path, sizeof path, "%s/%07d/state", c.P.caseFolder.c_str(), c.P.startStep);
    FILE *fp = fopen(path, "rb");
    if (!fp) throw InputError(std::string("restart: cannot open ") + path);
    auto S = state_arrays(c);
    char magic[8];
    int head[6];
    const bool ok = fread(magic, 1, 8, fp) == 8 && fread(head, sizeof(int), 6, fp) == 6 &&
                    std::equal(magic, magic + 8, kStateMagic) && head[0] == 1 && head[1] == c.g.nx &&
                    head[2] == c.g.ny && head[3] == c.P.startStep && head[4] == (c.has_body ? c.body.total : 0) &&
                    head[5] == (int)S.size();
    if (!ok) {
        fclose(fp);
        throw InputError(std::string("restart: ") + path + " does not hold this case's state at step " +
                         std::to_string(c.P.startStep));
    }
    std::vector<std::vector<double>> host;
    for (auto &a : S) {
        host.emplace_back(a.second);
        if (fread(host.back().data(), sizeof(double), a.second, fp) != a.second) {
            fclose(fp);
            throw InputError(std::string("restart: ") + path + " is truncated");
        }
    }
    fclose(fp);
    for (size_t k = 0; k < S.size(); ++k)
        CUIBM_TRY(cudaMemcpyAsync(S[k].first, host[k].data(), S[k].second * sizeof(double), cudaMemcpyHostToDevice,
                                  c.stream));
    CUIBM_TRY(cudaStreamSynchronize(c.stream));
}

void write_step_output(Context &c)
{
    if (!c.P.writeOutput) return;
    int it1 = 0, it2 = 0;
    read_solve_status(c, c.sys1, &it1);
    read_solve_status(c, c.sys2, &it2);
    if (c.iterationsFile) fprintf(c.iterationsFile, "%d\t%d\t%d\n", c.timeStep, it1, it2);
    if (c.timeStep % c.P.nsave == 0) {
        char dir[4096];
        snprintf(dir, sizeof dir, "%s/%07d", c.P.caseFolder.c_str(), c.timeStep);
        mkdir(dir, 0755);
        std::vector<double> q(c.g.nUV), lam(c.g.nP);
        CUIBM_TRY(cudaMemcpyAsync(q.data(), c.uhat, q.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        CUIBM_TRY(cudaMemcpyAsync(lam.data(), c.p, lam.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        CUIBM_TRY(cudaStreamSynchronize(c.stream));
        write_array(std::string(dir) + "/q", q);
        write_array(std::string(dir) + "/lambda", lam);
        write_restart_state(c, dir);
        if (c.has_body) {
            std::vector<double> bx(c.body.total), by(c.body.total);
            CUIBM_TRY(cudaMemcpyAsync(bx.data(), c.ib.bx, bx.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
            CUIBM_TRY(cudaMemcpyAsync(by.data(), c.ib.by, by.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
            CUIBM_TRY(cudaStreamSynchronize(c.stream));
            FILE *fp = fopen((std::string(dir) + "/bodies").c_str(), "w");
            if (fp) {
                fprintf(fp, "#%19s%20s\n", "x-coordinate", "y-coordinate");
                for (int l = 0; l < c.body.total; ++l) fprintf(fp, "%g\t%g\n", bx[l], by[l]);
                fclose(fp);
            }
        }
    }
    if (c.has_body) {
        double f[8] = {0, 0, 0, 0, 0, 0, 0, 0}, m[4] = {0, 0, 0, 0};
        CUIBM_TRY(cudaMemcpyAsync(f, c.ib.forceOut, sizeof f, cudaMemcpyDeviceToHost, c.stream));
        CUIBM_TRY(cudaMemcpyAsync(m, c.ib.motion, sizeof m, cudaMemcpyDeviceToHost, c.stream));
        CUIBM_TRY(cudaStreamSynchronize(c.stream));
        if (c.forceFile && c.P.solverType == ST_FADLUN) {
            // fadlunModified.cu:64-78: time, Fx and its three parts, Fy
            if (c.timeStep == 0) fprintf(c.forceFile, "timestep\tFx\tFxX\tFxY\tFxU\tFy\n");
            fprintf(c.forceFile, "%g\t%g\t%g\t%g\t%g\t%g\n", c.timeStep * c.P.dt, f[0], f[2], f[3], f[4], f[1]);
        } else if (c.forceFile) {
            if (c.timeStep == 1) fprintf(c.forceFile, "timestep\tFx\tFy\n");
            fprintf(c.forceFile, "%g\t%g\t%g\n", c.timeStep * c.P.dt, f[0], f[1]);
        }
        if (c.midPositionFile) {
            if (c.timeStep == 1) fprintf(c.midPositionFile, "ts\tX\tY\tU\tV\n");
            fprintf(c.midPositionFile, "%d\t%g\t%g\t%g\t%g\n", c.timeStep, m[0], m[1], m[2], m[3]);
        }
    }
    if (c.iterationsFile) fflush(c.iterationsFile);
}

}  // namespace cuibm
