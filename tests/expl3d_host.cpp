// Host build of the 3D explicit projection parts (pybella_gb300/csrc/bella_expl3d.cuh,
// with the advection's boundary lines) for tests/test_expl3d_host.py: the per-cell,
// per-node and per-line functions the kernels of bella_expl3d.cu run, in the same
// order, executed by loops.
#include "../pybella_gb300/csrc/bella_advect.cuh"
#include "../pybella_gb300/csrc/bella_expl3d.cuh"

using namespace bella;

namespace {

// ints: icx, icy, icz, walls[3], is_compressible, is_ArakawaKonor, div_sign_2d
// doubles: dx, dy, dz, dt, Msq, g, gamm, nonhydro, compressibility, cor[3], wind[3]
void setup(const int *gi, const double *gd, double **fields, Expl3Geom &G, Expl3Fields &F, AdvGeom &A,
           AdvFields &AF) {
    G.icx = gi[0]; G.icy = gi[1]; G.icz = gi[2];
    for (int q = 0; q < 3; ++q) G.bc[q] = gi[3 + q];
    G.is_ArakawaKonor = gi[7];
    G.xsign = gi[8] ? 1.0 : -1.0;
    G.dx = gd[0]; G.dy = gd[1]; G.dz = gd[2]; G.dt = gd[3];
    G.Msq = gd[4]; G.g = gd[5]; G.gamm = gd[6]; G.nonhydro = gd[7]; G.compressibility = gd[8];
    for (int q = 0; q < 3; ++q) {
        G.cor[q] = gd[9 + q];
        G.wind[q] = gd[12 + q];
    }
    for (int q = 0; q < 6; ++q) F.f[q] = AF.f[q] = fields[q];
    A.nd = 3;
    A.ic[0] = G.icx; A.ic[1] = G.icy; A.ic[2] = G.icz;
    for (int q = 0; q < 3; ++q) A.bc[q] = G.bc[q];
    A.d[0] = G.dx; A.d[1] = G.dy; A.d[2] = G.dz;
    A.g = G.g; A.gamm = G.gamm; A.is_compressible = gi[6];
}

void boundary(const AdvGeom &A, const AdvFields &AF, const double *rhoY0, const double *strat_inv) {
    for (int s = 0; s < 3; ++s)
        for (int l = 0; l < adv_nl(A, s); ++l) adv_bd_line(A, s, l, AF, rhoY0, strat_inv);
}

}  // namespace

extern "C" {

void e3_host_expl_part(const int *gi, const double *gd, double **fields, const double *S0n, const double *rhoY0,
                       const double *strat_inv) {
    Expl3Geom G; Expl3Fields F; AdvGeom A; AdvFields AF;
    setup(gi, gd, fields, G, F, A, AF);
    for (int i = 0; i < G.icx; ++i)
        for (int j = 0; j < G.icy; ++j)
            for (int k = 0; k < G.icz; ++k) e3_expl_part_cell(G, e3_cell(G, i, j, k), j, S0n, F);
    boundary(A, AF, rhoY0, strat_inv);
}

void e3_host_forward(const int *gi, const double *gd, double **fields, double *p2, double *rhs, double *dp,
                     const double *S0c, const double *S0n, const double *rhoY0, const double *strat_inv) {
    Expl3Geom G; Expl3Fields F; AdvGeom A; AdvFields AF;
    setup(gi, gd, fields, G, F, A, AF);
    if (G.bc[1] == 1)
        for (int i = 0; i < G.icx; ++i)
            for (int k = 0; k < G.icz; ++k) {
                const int rows[4] = {0, 1, G.icy - 2, G.icy - 1};
                for (int t = 0; t < 4; ++t)
                    for (int q = 1; q <= 3; ++q) F.f[q][e3_cell(G, i, rows[t], k)] = 0.0;
            }
    for (int a = 0; a < G.icx - 1; ++a)
        for (int b = 0; b < G.icy - 1; ++b)
            for (int c = 0; c < G.icz - 1; ++c) {
                const long long e = e3_isc(G, a, b, c);
                rhs[e] = e3_forward_node(G, a, b, c, F, &dp[e]);
            }
    for (int i = 0; i < G.icx; ++i)
        for (int j = 0; j < G.icy; ++j)
            for (int k = 0; k < G.icz; ++k) e3_forward_cell(G, i, j, k, p2, S0c, S0n, F);
    for (int a = 0; a < G.icx - 1; ++a)
        for (int b = 0; b < G.icy - 1; ++b)
            for (int c = 0; c < G.icz - 1; ++c) p2[e3_node(G, a + 1, b + 1, c + 1)] += G.compressibility * dp[e3_isc(G, a, b, c)];
    const long long nn[3] = {(long long)G.icx + 1, (long long)G.icy + 1, (long long)G.icz + 1};
    for (int d = 0; d < 3; ++d)
        for (long long l = 0; l < nn[d == 0 ? 1 : 0] * nn[d == 2 ? 1 : 2]; ++l) e3_ghost_line(G, d, l, p2);
    boundary(A, AF, rhoY0, strat_inv);
}

}
