// Host build of the double-float hydro pair formula (research_codes_gb300/csrc/hydro_df.cuh)
// for tests/test_hydro_df_host.py: one walk, every j but the i-particle itself, in one-pair or
// packed two-pair order, with the records built as make_hydro_records builds them.
#include <vector>
#include <cstring>
#include <cmath>
#include <vector_types.h>
#include <vector_functions.h>
#include "../research_codes_gb300/csrc/hydro_df.cuh"
using namespace sphk;
static float2 split(double v) { float h = (float)v; return make_float2(h, (float)(v - (double)h)); }
// One particle's FP32C hydro records from its 17 FP64 fields:
// x y z vx vy vz m hinv pres presc bswt dens vsnd alph alphu thrm eta.
static HydroDFP<float> mk(const double *r) {
    float2 x = split(r[0]), y = split(r[1]), z = split(r[2]), u = split(r[3]), w = split(r[4]), s = split(r[5]);
    float2 P = split(r[8]), T = split(r[15]), Q = split(r[9]);
    double h4d = (r[7] * r[7]) * (r[7] * r[7]);
    float2 H = split(r[7]), H4 = split(h4d), M = split(r[6]);
    float4 phi = make_float4(x.x, y.x, z.x, M.x), plo = make_float4(x.y, y.y, z.y, M.y);
    float4 vhi = make_float4(u.x, w.x, s.x, H.x), vlo = make_float4(u.y, w.y, s.y, H4.x);
    float4 g1 = make_float4(P.x, P.y, Q.x, (float)r[10]);
    float4 g2 = make_float4((float)r[11], (float)r[12], (float)r[13], (float)r[14]);
    float4 g3 = make_float4(T.x, T.y, (float)r[16], Q.y);
    float4 g4 = make_float4(H.x, H.y, H4.x, H4.y);
    return hydro_df_rec(phi, plo, vhi, vlo, g1, g2, g3, g4);
}
extern "C" void df_walk(int ni, const double *ri, const long long *idi, int nj, const double *rj, const long long *idj,
                        int packed, double *out /* 8 per i: acch[3] accg[3] udot diffu */) {
    const double c1 = 1.336901521971920914e+01;
    for (int a = 0; a < ni; ++a) {
        HydroDFP<float> I = mk(ri + 17 * a);
        HydroDFAcc<float> acc = hydro_df_zero<float>();
        std::vector<int> js;
        for (int b = 0; b < nj; ++b) if (idj[b] != idi[a]) js.push_back(b);
        int k = 0;
        if (packed) {
            HydroDFP<dfk::pk> I2 = hydro_df_pack(I, I);
            HydroDFAcc<dfk::pk> acc2 = hydro_df_zero<dfk::pk>();
            for (; k + 1 < (int)js.size(); k += 2)
                hydro_df_pair(I2, hydro_df_pack(mk(rj + 17 * js[k]), mk(rj + 17 * js[k + 1])), acc2);
            if (k < (int)js.size()) hydro_df_pair(I, mk(rj + 17 * js[k]), acc);
            dfk::df *v[9] = {&acc.ax, &acc.ay, &acc.az, &acc.gx, &acc.gy, &acc.gz, &acc.ud, &acc.uv, &acc.dif};
            dfk::dv<dfk::pk> *w[9] = {&acc2.ax, &acc2.ay, &acc2.az, &acc2.gx, &acc2.gy, &acc2.gz, &acc2.ud, &acc2.uv, &acc2.dif};
            for (int q = 0; q < 9; ++q) *v[q] = dfk::add(dfk::add(lane0(*w[q]), lane1(*w[q])), *v[q]);
        } else {
            for (int b : js) hydro_df_pair(I, mk(rj + 17 * b), acc);
        }
        double *o = out + 8 * a;
        hydro_df_finish(acc, I.presc, c1, o, o + 3, o + 6, o + 7);
    }
}
