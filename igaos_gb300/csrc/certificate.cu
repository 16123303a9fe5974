// Infeasibility certificates (host code; see certificate.hpp). No counterpart
// in the reference engine, which ends an LP without a solution at its cap.
#include "certificate.hpp"

#include <algorithm>
#include <cmath>

namespace igx {

int ray_certificate(int m, int n, const double* x, const double* ax, const double* y,
                    const double* aty, const double* c, const double* cl, const double* cu,
                    const double* rmin, const double* rmax, double* xray, double* yray) {
    double ymax = 0.0, xmax = 0.0;
    for (int i = 0; i < m; ++i) ymax = std::max(ymax, std::fabs(y[i]));
    for (int j = 0; j < n; ++j) xmax = std::max(xmax, std::fabs(x[j]));
    if (ymax > 0.0 && std::isfinite(ymax)) {  // dual ray
        double obj = 0.0, mag = 0.0, viol = 0.0, dmax = 0.0;
        for (int j = 0; j < n; ++j) {
            const double d = aty[j] / ymax;
            dmax = std::max(dmax, std::fabs(d));
            if (d > 0.0) {
                if (std::isfinite(cl[j])) {
                    obj += d * cl[j];
                    mag += std::fabs(d * cl[j]);
                } else {
                    viol = std::max(viol, d);
                }
            } else if (d < 0.0) {
                if (std::isfinite(cu[j])) {
                    obj += d * cu[j];
                    mag += std::fabs(d * cu[j]);
                } else {
                    viol = std::max(viol, -d);
                }
            }
        }
        for (int i = 0; i < m; ++i) {
            const double v = y[i] / ymax;
            if (v > 0.0) {
                if (std::isfinite(rmax[i])) {
                    obj -= v * rmax[i];
                    mag += std::fabs(v * rmax[i]);
                } else {
                    viol = std::max(viol, v);
                }
            } else if (v < 0.0) {
                if (std::isfinite(rmin[i])) {
                    obj -= v * rmin[i];
                    mag += std::fabs(v * rmin[i]);
                } else {
                    viol = std::max(viol, -v);
                }
            }
        }
        if (obj > 0.0 && obj > kRayObjRel * mag && viol <= kRayViolRel * std::max(1.0, dmax)) {
            if (yray)
                for (int i = 0; i < m; ++i) yray[i] = y[i] / ymax;
            return 1;
        }
    }
    if (xmax > 0.0 && std::isfinite(xmax)) {  // primal ray
        double cx = 0.0, mag = 0.0, viol = 0.0, amax = 0.0;
        for (int j = 0; j < n; ++j) {
            const double v = x[j] / xmax;
            cx += c[j] * v;
            mag += std::fabs(c[j] * v);
            if (v < 0.0 && std::isfinite(cl[j])) viol = std::max(viol, -v);
            if (v > 0.0 && std::isfinite(cu[j])) viol = std::max(viol, v);
        }
        for (int i = 0; i < m; ++i) {
            const double a = ax[i] / xmax;
            amax = std::max(amax, std::fabs(a));
            if (a < 0.0 && std::isfinite(rmin[i])) viol = std::max(viol, -a);
            if (a > 0.0 && std::isfinite(rmax[i])) viol = std::max(viol, a);
        }
        if (cx < 0.0 && -cx > kRayObjRel * mag && viol <= kRayViolRel * std::max(1.0, amax)) {
            if (xray)
                for (int j = 0; j < n; ++j) xray[j] = x[j] / xmax;
            return 2;
        }
    }
    return 0;
}

}  // namespace igx
