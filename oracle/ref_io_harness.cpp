/*
 * Host entry points around the reference's own grid and body parsers
 * (io/parseDomainFile.cu, io/parseBodiesFile.cu), TEST INFRASTRUCTURE ONLY.
 *
 * oracle/Makefile compiles those two reference files in place with
 * oracle/ref_include first on the include path (stand-ins for CUSP's array1d,
 * yaml-cpp and parameterDB) and links them with this file.  The case files are
 * given as JSON with the same tree as the YAML the product reads.
 */
#include <cstring>
#include <string>
#include <vector>
#include <domain.h>
#include <body.h>
#include <parameterDB.h>

namespace io {
void parseDomainFile(std::string &domFile, domain &D);
void parseBodiesFile(std::string &bodiesFile, parameterDB &DB);
}  // namespace io

static std::vector<body> g_bodies;
std::vector<body> *ref_body_list() { return &g_bodies; }
static domain g_domain;

extern "C" {
int ref_parse_domain(const char *json_path, int *nx, int *ny, double *mid_h)
{
    std::string f(json_path);
    g_domain = domain();
    io::parseDomainFile(f, g_domain);
    *nx = g_domain.nx;
    *ny = g_domain.ny;
    *mid_h = g_domain.mid_h;
    return 0;
}

void ref_domain_arrays(double *x, double *dx, double *xu, double *xv, double *y, double *dy, double *yu,
                       double *yv)
{
    const domain &D = g_domain;
    std::memcpy(x, D.x.data(), sizeof(double) * D.nx);
    std::memcpy(dx, D.dx.data(), sizeof(double) * D.nx);
    std::memcpy(xu, D.xu.data(), sizeof(double) * (D.nx - 1));
    std::memcpy(xv, D.xv.data(), sizeof(double) * D.nx);
    std::memcpy(y, D.y.data(), sizeof(double) * D.ny);
    std::memcpy(dy, D.dy.data(), sizeof(double) * D.ny);
    std::memcpy(yu, D.yu.data(), sizeof(double) * D.ny);
    std::memcpy(yv, D.yv.data(), sizeof(double) * (D.ny - 1));
}

int ref_parse_bodies(const char *json_path, int *numBodies)
{
    std::string f(json_path);
    parameterDB DB;
    g_bodies.clear();
    io::parseBodiesFile(f, DB);
    *numBodies = (int)g_bodies.size();
    return 0;
}

// numPoints of body k, then its reference coordinates X, Y and the motion coefficients
int ref_body_numpoints(int k) { return g_bodies[k].numPoints; }
void ref_body_points(int k, double *X, double *Y, double *coef)
{
    const body &b = g_bodies[k];
    for (int i = 0; i < b.numPoints; ++i) { X[i] = b.X[i]; Y[i] = b.Y[i]; }
    coef[0] = b.xCoefficient; coef[1] = b.yCoefficient; coef[2] = b.uCoefficient; coef[3] = b.vCoefficient;
    coef[4] = b.xfrequency;   coef[5] = b.yfrequency;   coef[6] = b.xPhase;       coef[7] = b.yPhase;
    coef[8] = b.uPhase;       coef[9] = b.vPhase;
}
}
