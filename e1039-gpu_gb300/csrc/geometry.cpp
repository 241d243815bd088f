// geometry.cpp -- detector geometry loader for the C-ABI.
//
// Reads the plain-text geometry table (27 numeric columns per plane plus the
// wire offsets) into an or_plane_t, derives the LR-resolution slope and
// intercept windows and the wire-position table.  It follows the reference
// host (OnlineReconstruction/online_reconstruction.cu:123-218) so that the
// geometry handed to the kernels is byte-identical to the reference's:
//   - fields are extracted with `istream >> float`, so glued columns such as
//     "2.749630657183.4666022" split where a float literal ends;
//   - slope_max/inter_max get the pairwise resolution widening on even planes
//     (online_reconstruction.cu:177-186), summed in double;
//   - wire positions are computed in double (chambers, hodoscopes, prop-tube
//     modules with their own offset) and narrowed to float when hits are
//     packed.
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>

#include "../../include/or_gb300.h"

extern "C" int or_geometry_load(const char *path, or_plane_t *plane, double *wire_pos) {
    if (!path || !plane) return OR_ERR_ARG;
    std::ifstream in(path);
    if (!in) return OR_ERR_IO;
    std::memset(plane, 0, sizeof(*plane));
    const float tx_max = 0.15f, ty_max = 0.1f, x0_max = 150.f, y0_max = 50.f;
    float deltaw[OR_NDET][9];
    std::memset(deltaw, 0, sizeof(deltaw));

    std::string line;
    int ipl = 0, nelem = 0;
    float v[25] = {0};
    float dw = 0.f;
    int nplanes = 0;
    while (std::getline(in, line)) {
        if (!line.empty() && line[0] == '#') continue;
        if (line.empty()) continue;
        std::istringstream is(line);
        float z = 0.f;
        is >> ipl >> z >> nelem;
        for (int k = 0; k < 23; ++k) is >> v[k];
        if (ipl < 1 || ipl >= OR_NDET) continue;
        plane->z[ipl] = z;
        plane->nelem[ipl] = nelem;
        float *dst[23] = {&plane->cellwidth[ipl], &plane->spacing[ipl], &plane->xoffset[ipl], &plane->scalex[ipl],
                          &plane->x0[ipl],        &plane->x1[ipl],      &plane->x2[ipl],      &plane->costheta[ipl],
                          &plane->scaley[ipl],    &plane->y0[ipl],      &plane->y1[ipl],      &plane->y2[ipl],
                          &plane->sintheta[ipl],  &plane->resolution[ipl], &plane->p1x_w1[ipl], &plane->p1y_w1[ipl],
                          &plane->p1z_w1[ipl],    &plane->deltapx[ipl], &plane->deltapy[ipl], &plane->deltapz[ipl],
                          &plane->dp1x[ipl],      &plane->dp1y[ipl],    &plane->dp1z[ipl]};
        for (int k = 0; k < 23; ++k) *dst[k] = v[k];
        const int nw = (ipl > OR_NCHAM + OR_NHODO) ? 9 : 1;
        for (int k = 0; k < nw; ++k) {
            is >> dw;  // a missing column leaves the previous value, as `>>` does
            deltaw[ipl][k] = dw;
        }
        const float c = plane->costheta[ipl], s = plane->sintheta[ipl];
        plane->slope_max[ipl] = c * tx_max + s * ty_max;
        plane->inter_max[ipl] = c * x0_max + s * y0_max;
        if (ipl % 2 == 0 && ipl > 1) {
            const float num = plane->resolution[ipl] + plane->resolution[ipl - 1];
            const float den = plane->z[ipl] - plane->z[ipl - 1];
            const double dslope = static_cast<double>(num / den);
            const double dinter = dslope * static_cast<double>(plane->z[ipl]);
            plane->slope_max[ipl] = static_cast<float>(plane->slope_max[ipl] + dslope);
            plane->inter_max[ipl] = static_cast<float>(plane->inter_max[ipl] + dinter);
            plane->slope_max[ipl - 1] = static_cast<float>(plane->slope_max[ipl - 1] + dslope);
            plane->inter_max[ipl - 1] = static_cast<float>(plane->inter_max[ipl - 1] + dinter);
        }
        ++nplanes;
    }
    if (nplanes == 0) return OR_ERR_IO;

    if (wire_pos) {
        for (int i = 0; i < OR_NDET * OR_WIREPOS_STRIDE; ++i) wire_pos[i] = 0.0;
        for (int i = 1; i < OR_NDET; ++i) {
            const int n = plane->nelem[i];
            for (int j = 1; j <= n && j < OR_WIREPOS_STRIDE; ++j) {
                double pos;
                if (i <= OR_NCHAM) {
                    // chambers: offset terms added one by one in double
                    pos = (j - (n + 1.) / 2.) * plane->spacing[i];
                    pos += plane->xoffset[i];
                    pos += static_cast<float>(plane->x0[i] * plane->costheta[i]);
                    pos += static_cast<float>(plane->y0[i] * plane->sintheta[i]);
                    pos += deltaw[i][0];
                } else {
                    // hodoscopes and prop tubes: the float terms are summed in
                    // float first; prop tubes take one offset per 8-tube module
                    float f = plane->x0[i] * plane->costheta[i];
                    f = f + plane->y0[i] * plane->sintheta[i];
                    f = f + plane->xoffset[i];
                    pos = static_cast<double>(f) + (j - (n + 1) / 2.) * plane->spacing[i];
                    const int module = (i > OR_NCHAM + OR_NHODO) ? 8 - (j - 1) / 8 : 0;
                    pos += deltaw[i][module];
                }
                wire_pos[i * OR_WIREPOS_STRIDE + j] = pos;
            }
        }
    }
    return OR_OK;
}
