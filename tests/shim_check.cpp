// Compiles include/gb_projectors.H the way incflo would use it and runs one small nodal projection
// (16^3, periodic x/y, walls in z) through the C ABI. Without a usable GPU it must report
// GBP_NO_DEVICE cleanly (exit code 3) instead of aborting. Exit codes: 0 ok, 1 wrong result,
// 2 unexpected error, 3 no device.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>

#include <vector>

#include "gb_projectors.H"

int main()
{
    const int n = 16, g = 1;
    const int lo[3] = {-g, -g, -g}, hi[3] = {n - 1 + g, n - 1 + g, n - 1 + g};
    const int clo[3] = {0, 0, 0}, chi[3] = {n - 1, n - 1, n - 1};
    const int nlo[3] = {0, 0, 0}, nhi[3] = {n, n, n};
    const size_t nv = 3 * (size_t)(n + 2) * (n + 2) * (n + 2);
    const size_t nc = (size_t)n * n * n, nn = (size_t)(n + 1) * (n + 1) * (n + 1);
    try {
        gb::Geometry geom{{n, n, n}, {0, 0, 0}, {1, 1, 1}};
        int dev_ok = gbp_device_check();
        if (dev_ok != GBP_OK) {
            // the shim must surface the status, not abort
            gb::NodalProjector probe(gbp_array4{}, 1.0, geom);
            const int bl[3] = {GBP_BC_PERIODIC, GBP_BC_PERIODIC, GBP_BC_NEUMANN};
            try {
                probe.setDomainBC(bl, bl);
            } catch (const gb::Error& e) {
                printf("no device: %s\n", e.what());
                return e.status == GBP_NO_DEVICE ? 3 : 2;
            }
            return 2;
        }
        std::vector<double> hv(nv, 0.0), hs(nc);
        for (size_t i = 0; i < nv; ++i) hv[i] = sin(0.37 * (double)i) * cos(0.011 * (double)i);
        for (size_t i = 0; i < nc; ++i) hs[i] = 0.5 + 0.25 * sin(0.7 * (double)i);
        double *dv, *ds, *dp, *dg;
        cudaMalloc(&dv, nv * 8);
        cudaMalloc(&ds, nc * 8);
        cudaMalloc(&dp, nn * 8);
        cudaMalloc(&dg, 3 * nc * 8);
        cudaMemcpy(dv, hv.data(), nv * 8, cudaMemcpyHostToDevice);
        cudaMemcpy(ds, hs.data(), nc * 8, cudaMemcpyHostToDevice);
        gb::NodalProjector proj(gb::view(dv, lo, hi, 3), gb::view(ds, clo, chi), geom, gb::LPInfo{}, nullptr,
                                "nodal_proj.mg_rtol = 1e-12\nnodal_proj.mg_atol = 0\n");
        const int bl[3] = {GBP_BC_PERIODIC, GBP_BC_PERIODIC, GBP_BC_NEUMANN};
        proj.setDomainBC(bl, bl);
        proj.setOutputs(gb::view(dp, nlo, nhi), gb::view(dg, clo, chi, 3));
        gbp_stats st = proj.project(1e-12, 0.0);
        printf("status %d vcycles %d rel resid %.3e\n", st.status, st.vcycles, st.final_rel_resid);
        cudaFree(dv);
        cudaFree(ds);
        cudaFree(dp);
        cudaFree(dg);
        return (st.status == GBP_OK && st.final_rel_resid <= 1e-12) ? 0 : 1;
    } catch (const gb::Error& e) {
        printf("error: %s\n", e.what());
        return 2;
    }
}
