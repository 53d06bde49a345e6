// Test shim (CPU): the host parse of the GALWIND stream (bbh_wind_clouds) with its arrays copied out, so that the
// CPU tests compare it with the oracle's stream without a GPU.
#include <string.h>

#include "../../bbarolo2_gb300/csrc/internal.h"

extern "C" int wind_clouds_dump(uint64_t seed, const double *sr, int nsub, int lo, int hi, double sep,
                                const int64_t *nv, double cdens, int cmode, double pixarea, double sig_instr,
                                double crota2, long long *counts, double *shells, int *shell, double *geo,
                                long long *nbase, long long *sbase, int *hz, double *slow) {
    GridDev g{};
    g.cdens = cdens;
    g.cmode = cmode;
    g.pixarea = pixarea;
    g.sig_instr = sig_instr;
    g.crota2 = crota2;
    WindClouds W;
    const int e = bbh_wind_clouds(&W, seed, sr, nsub, lo, hi, sep, nv, &g);
    if (e) return e;
    counts[0] = (long long)W.shells.size();
    counts[1] = (long long)W.shell.size();
    counts[2] = (long long)W.hz.size();
    counts[3] = (long long)W.slow.size();
    if (shells) memcpy(shells, W.shells.data(), sizeof(WindShell) * W.shells.size());
    if (shell) memcpy(shell, W.shell.data(), sizeof(int) * W.shell.size());
    if (geo) memcpy(geo, W.geo.data(), sizeof(double) * W.geo.size());
    if (nbase) memcpy(nbase, W.nbase.data(), sizeof(long long) * W.nbase.size());
    if (sbase) memcpy(sbase, W.sbase.data(), sizeof(long long) * W.sbase.size());
    if (hz) memcpy(hz, W.hz.data(), sizeof(int) * W.hz.size());
    if (slow) memcpy(slow, W.slow.data(), sizeof(double) * W.slow.size());
    return 0;
}
