// Starting states of the reference's own LLE map, for parity on identical
// inputs. Compiles the reference's unchanged LLE/src/LLECUDA.cu into this
// program (staged by oracle/build_ref_gpu.py, Rossler RK4 plug-in as its
// systems.cuh), sets the constants its LLE2D host driver sets
// (LLE/src/LLECUDA.cu:260-292) for one segment, and launches its two kernels
// as LLE2D launches them (LLECUDA.cu:337-369): calculateTransTime (the
// transient, then the twin start from its cuRAND draw, rounded through FP32)
// and calculateSystem (the Benettin blocks). Writes the semi_result rows the
// first kernel left and the map the second computed from them.
// TEST INFRASTRUCTURE ONLY: never shipped, never called by the engine.
//
//   ref_gpu_lle_states <out.bin> [nPts] [tMax]
//
// out.bin: int32 nPts, int32 W (= 2*SIZE_X + SIZE_A), then nPts*nPts rows of
// W doubles at row (ia*nPts + ib) -- the reference's semi_result indexing,
// ia the index of the first swept parameter, ib of the second -- then the
// nPts*nPts map values at (ia*nPts + ib) (its result[ia][ib]).
#include "LLECUDA.cu"

#include <cstdio>
#include <cstdlib>
#include <vector>

using namespace LLE_constants;

#define CK(x)                                                                  \
    do {                                                                       \
        cudaError_t e_ = (x);                                                  \
        if (e_ != cudaSuccess) {                                               \
            fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(e_));           \
            return 1;                                                          \
        }                                                                      \
    } while (0)

int main(int argc, char** argv) {
    const char* path = argc > 1 ? argv[1] : "ref_states.bin";
    const int nPts = argc > 2 ? atoi(argv[2]) : 128;
    const double tMax = argc > 3 ? atof(argv[3]) : 500.0;
    if (nPts < 2 || nPts > 1024) {
        fprintf(stderr, "nPts must be in [2, 1024]\n");
        return 2;
    }
    // the benchmark's LLE map (Rossler, a in [0.1, 0.4], c in [2, 10])
    const double h = 0.01, NT = 0.1, eps = 1e-8, transientTime = 50.0;
    const double ic[3] = {1.0, 1.0, 1.0}, ranges[4] = {0.1, 0.4, 2.0, 10.0}, values[3] = {0.2, 0.2, 5.7};
    const int mut[2] = {0, 2}, nX = 3, nA = 3, W = 2 * nX + nA;

    const int ntPoints = static_cast<int>(NT / h);
    const int transPoints = static_cast<int>(transientTime / h);
    const int allPoints = static_cast<int>(tMax / h);
    const int calcBlocks = allPoints / ntPoints + 1;
    CK(cudaMemcpyToSymbol(d_idxParamA, &mut[0], sizeof(int)));
    CK(cudaMemcpyToSymbol(d_idxParamB, &mut[1], sizeof(int)));
    CK(cudaMemcpyToSymbol(d_size_linspace_A, &nPts, sizeof(int)));
    CK(cudaMemcpyToSymbol(d_size_linspace_B, &nPts, sizeof(int)));
    CK(cudaMemcpyToSymbol(d_h, &h, sizeof(double)));
    CK(cudaMemcpyToSymbol(d_transTime, &transientTime, sizeof(double)));
    CK(cudaMemcpyToSymbol(d_tMax, &tMax, sizeof(double)));
    CK(cudaMemcpyToSymbol(d_Nt_steps, &ntPoints, sizeof(int)));
    CK(cudaMemcpyToSymbol(d_paramsSize, &nA, sizeof(int)));
    CK(cudaMemcpyToSymbol(d_XSize, &nX, sizeof(int)));
    CK(cudaMemcpyToSymbol(d_amountOfNTPoints, &ntPoints, sizeof(int)));
    CK(cudaMemcpyToSymbol(d_amountOfTransPoints, &transPoints, sizeof(int)));
    CK(cudaMemcpyToSymbol(d_amountOfAllpoints, &allPoints, sizeof(int)));
    CK(cudaMemcpyToSymbol(d_amountOfCalcBlocks, &calcBlocks, sizeof(int)));
    const double h1 = values[0] * h, h2 = (1 - values[0]) * h;
    CK(cudaMemcpyToSymbol(d_h1, &h1, sizeof(double)));
    CK(cudaMemcpyToSymbol(d_h2, &h2, sizeof(double)));
    CK(cudaMemcpyToSymbol(d_eps, &eps, sizeof(double)));

    double* linA = linspace(ranges[0], ranges[1], nPts);  // the reference's own host linspace
    double* linB = linspace(ranges[2], ranges[3], nPts);
    const size_t n = (size_t)nPts * nPts;
    double *dSemi, *dLinA, *dLinB, *dIc, *dVal;
    CK(cudaMalloc(&dSemi, n * W * sizeof(double)));
    CK(cudaMalloc(&dLinA, nPts * sizeof(double)));
    CK(cudaMalloc(&dLinB, nPts * sizeof(double)));
    CK(cudaMalloc(&dIc, nX * sizeof(double)));
    CK(cudaMalloc(&dVal, nA * sizeof(double)));
    CK(cudaMemcpy(dLinA, linA, nPts * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dLinB, linB, nPts * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dIc, ic, nX * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dVal, values, nA * sizeof(double), cudaMemcpyHostToDevice));
    // result rows, one per first-parameter index, zeroed (its kernel adds into them)
    std::vector<double*> rows(nPts);
    double* dRowsAll;
    double** dRows;
    CK(cudaMalloc(&dRowsAll, n * sizeof(double)));
    CK(cudaMemset(dRowsAll, 0, n * sizeof(double)));
    for (int i = 0; i < nPts; ++i) rows[i] = dRowsAll + (size_t)i * nPts;
    CK(cudaMalloc(&dRows, nPts * sizeof(double*)));
    CK(cudaMemcpy(dRows, rows.data(), nPts * sizeof(double*), cudaMemcpyHostToDevice));

    const dim3 block(16, 16, 1), grid((nPts + 15) / 16, (nPts + 15) / 16, 1);
    const size_t shmem = 16 * 16 * W * sizeof(double);
    calculateTransTime<<<grid, block, shmem>>>(dIc, dVal, dLinA, dLinB, dSemi);
    CK(cudaDeviceSynchronize());
    CK(cudaPeekAtLastError());
    calculateSystem<<<grid, block, shmem>>>(dIc, dVal, dLinA, dLinB, dSemi, dRows);
    CK(cudaDeviceSynchronize());
    CK(cudaPeekAtLastError());

    std::vector<double> semi(n * W), res(n);
    CK(cudaMemcpy(semi.data(), dSemi, semi.size() * sizeof(double), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(res.data(), dRowsAll, n * sizeof(double), cudaMemcpyDeviceToHost));
    FILE* f = fopen(path, "wb");
    if (!f) {
        fprintf(stderr, "cannot open %s\n", path);
        return 1;
    }
    const int hdr[2] = {nPts, W};
    fwrite(hdr, sizeof(int), 2, f);
    fwrite(semi.data(), sizeof(double), semi.size(), f);
    fwrite(res.data(), sizeof(double), res.size(), f);
    fclose(f);
    delete[] linA;
    delete[] linB;
    printf("{\"nPts\": %d, \"W\": %d}\n", nPts, W);
    return 0;
}
