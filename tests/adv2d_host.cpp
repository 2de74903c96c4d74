// Host build of the device advection arithmetic (pybella_gb300/csrc/bella_adv2d.cuh)
// for tests/test_adv2d_host.py: the same per-face, per-cell and per-line functions
// and the same sweep sequences the kernels of bella_adv2d.cu run, executed by loops,
// so their arithmetic and indexing are checked against the oracle without a GPU.
#include "../pybella_gb300/csrc/bella_adv2d.cuh"

using namespace bella;

namespace {

struct HostEx {
    AdvGeom G;
    AdvFields F;
    AdvFaces fl[2];
    const double *rhoY0, *strat_inv;
    double *pw;
    void bd(int s) {
        for (int l = 0; l < adv_nl(G, s); ++l) adv_bd_line(G, s, l, F, rhoY0, strat_inv);
    }
    void faces(int s, double lmbda) {
        for (int l = 0; l < adv_nl(G, s); ++l)
            for (int f = 1; f <= adv_ns(G, s) - 1; ++f) adv_face_flux(G, s, l, f, F, lmbda, fl[s]);
    }
    void update(int s, double lmbda) {
        for (int l = 0; l < adv_nl(G, s); ++l)
            for (int c = 0; c < adv_ns(G, s); ++c) adv_update_cell(G, s, l, c, F, fl[s], lmbda);
    }
    void pwchi(double lmbda) {
        if (!pw) return;
        for (int l = 0; l < G.icx; ++l)
            for (int c = 0; c < G.icy; ++c)
                pw[adv_cell(G, 1, l, c)] = lmbda * (fl[1].f[5][adv_face(G, 1, l, c)] - fl[1].f[5][adv_face(G, 1, l, c + 1)]);
    }
};

HostEx make(int icx, int icy, int xw, int yw, double dx, double dy, double g, double gamm, int comp,
            double **fields, double **fx, double **fy, const double *rhoY0, const double *strat_inv, double *pw) {
    HostEx ex;
    ex.G.icx = icx; ex.G.icy = icy; ex.G.bc[0] = xw; ex.G.bc[1] = yw;
    ex.G.dx = dx; ex.G.dy = dy; ex.G.g = g; ex.G.gamm = gamm; ex.G.is_compressible = comp;
    for (int q = 0; q < 6; ++q) {
        ex.F.f[q] = fields[q];
        ex.fl[0].f[q] = fx[q];
        ex.fl[1].f[q] = fy[q];
    }
    ex.rhoY0 = rhoY0; ex.strat_inv = strat_inv; ex.pw = pw;
    return ex;
}

}  // namespace

extern "C" {

void adv_host_mass(int icx, int icy, double **fields, double *fx_rhoY, double *fy_rhoY) {
    AdvGeom G{};
    G.icx = icx; G.icy = icy;
    AdvFields F;
    for (int q = 0; q < 6; ++q) F.f[q] = fields[q];
    for (int j = 1; j <= icy - 2; ++j)
        for (int f = 1; f <= icx - 1; ++f) fx_rhoY[adv_face(G, 0, j, f)] = adv_mass_x(G, F, j, f);
    for (int i = 1; i <= icx - 2; ++i)
        for (int f = 1; f <= icy - 1; ++f) fy_rhoY[adv_face(G, 1, i, f)] = adv_mass_y(G, F, i, f);
}

void adv_host_strang(int icx, int icy, int xw, int yw, double dx, double dy, double g, double gamm, int comp,
                     double **fields, double **fx, double **fy, const double *rhoY0, const double *strat_inv,
                     double dt, int odd) {
    HostEx ex = make(icx, icy, xw, yw, dx, dy, g, gamm, comp, fields, fx, fy, rhoY0, strat_inv, nullptr);
    adv_strang(ex, ex.G, dt, odd);
}

void adv_host_rk(int icx, int icy, int xw, int yw, double dx, double dy, double g, double gamm, int comp,
                 double **fields, double **fx, double **fy, const double *rhoY0, const double *strat_inv, double dt,
                 double *pwchi) {
    HostEx ex = make(icx, icy, xw, yw, dx, dy, g, gamm, comp, fields, fx, fy, rhoY0, strat_inv, pwchi);
    adv_rk(ex, ex.G, dt);
}

}
