// main_dropin.cpp -- the reference's main.cu call sequence (src/main.cu:14-322)
// written against fastload_compat.h, to show the library drops in under it.
// Reads a CSR matrix from a small binary file (int32 m, n, nnz; rowptr;
// colidx) instead of a .mtx, then does what main.cu does: values i%10,
// csr_to_csc, x = i%10, CSR and CSC goldens, ColSort, formatTransform, the
// tile-order CPU check, FastLoad_spmv against the CSR golden, Tile_destroy.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "fastload_compat.h"

int main(int argc, char **argv) {
    if (argc < 2) {
        printf("error order\n");
        return 2;
    }
    int rowA = 0, colA = 0, nnz = 0;
    std::vector<int> csrrowptr, csrcolidx;
    const size_t len = strlen(argv[1]);
    if (len > 4 && strcmp(argv[1] + len - 4, ".mtx") == 0) {
        // main.cu:40, with the entries parsed on the GPU
        int isSymmetricA = 0, *rp = nullptr, *ci = nullptr;
        double *v = nullptr;
        if (mmio_allinone_gpu(&rowA, &colA, &nnz, &isSymmetricA, &rp, &ci, &v, argv[1]) != 0) return 3;
        csrrowptr.assign(rp, rp + rowA + 1);
        csrcolidx.assign(ci, ci + nnz);
        free(rp);
        free(ci);
        free(v);
    } else {
        FILE *f = fopen(argv[1], "rb");
        if (!f) return 2;
        int hdr[3];
        if (fread(hdr, sizeof(int), 3, f) != 3) return 2;
        rowA = hdr[0];
        colA = hdr[1];
        nnz = hdr[2];
        csrrowptr.resize(rowA + 1);
        csrcolidx.resize(nnz);
        if (fread(csrrowptr.data(), sizeof(int), rowA + 1, f) != (size_t)rowA + 1) return 2;
        if (fread(csrcolidx.data(), sizeof(int), nnz, f) != (size_t)nnz) return 2;
        fclose(f);
    }
    std::vector<double> csrval(nnz);
    for (int i = 0; i < nnz; i++) csrval[i] = i % 10;  // main.cu:68-69
    printf("read success,input matrix A :(%i,%i) nnz =%i  \n", rowA, colA, nnz);

    std::vector<int> cscrowidx(nnz), csccolptr(colA + 1), nnzpercol(colA);
    std::vector<double> cscval(nnz);
    double csr2cscTime = 0;
    csr_to_csc(csr2cscTime, rowA, colA, nnz, csrval.data(), csrrowptr.data(), csrcolidx.data(), cscval.data(),
               cscrowidx.data(), csccolptr.data(), nnzpercol.data());

    std::vector<double> x(colA);
    for (int i = 0; i < colA; i++) x[i] = i % 10;  // main.cu:93-96
    std::vector<double> y_goldencsr(rowA, 0.0), y_goldencsc(rowA, 0.0);
    for (int i = 0; i < rowA; i++) {
        double sum = 0;
        for (int j = csrrowptr[i]; j < csrrowptr[i + 1]; j++) sum += csrval[j] * x[csrcolidx[j]];
        y_goldencsr[i] = sum;
    }
    for (int i = 0; i < colA; i++)
        for (int j = csccolptr[i]; j < csccolptr[i + 1]; j++) y_goldencsc[cscrowidx[j]] += cscval[j] * x[i];
    int error_count_check = 0;
    for (int i = 0; i < rowA; i++)
        if (y_goldencsc[i] != y_goldencsr[i]) error_count_check++;
    if (error_count_check != 0) printf("Check NO PASS! error_count_check_csc_csr= %d \n", error_count_check);

    slide_matrix *matrixA = (slide_matrix *)malloc(sizeof(slide_matrix));
    std::vector<int> sortrowidx_tmp(nnz), sortnnz_tmp(colA);
    std::vector<double> sortval_tmp(nnz), sortx(colA);
    double timeForSort = 0;
    ColSort(timeForSort, rowA, colA, nnz, nnzpercol.data(), csccolptr.data(), cscrowidx.data(), cscval.data(),
            sortrowidx_tmp.data(), sortval_tmp.data(), sortnnz_tmp.data(), x.data(), sortx.data());
    int h_count = 0;
    double timeFormatTran = 0, timeFortmatClas = 0;
    formatTransform(timeFormatTran, timeFortmatClas, matrixA, sortrowidx_tmp.data(), sortval_tmp.data(),
                    sortnnz_tmp.data(), nnz, rowA, colA, h_count);
    printf("steps %d tilenum %d segsum %d\n", h_count, matrixA->tilenum, matrixA->segsum);

    // tile-order CPU pass over the layout, compared exactly (FastLoad_CPU.h:19-44)
    std::vector<double> y(rowA, 0.0);
    for (int i = 0; i < matrixA->tilenum; i++) {
        int start = matrixA->tile_ptr[i], stop = matrixA->tile_ptr[i + 1], len = matrixA->tile_len[i];
        for (int j = start; j < stop; j++)
            y[matrixA->sortrowidx[j]] += matrixA->sortval[j] * sortx[matrixA->tile_colidx[i] + (j - start) % len];
    }
    int error_count_check_cpu = 0;
    for (int i = 0; i < rowA; i++)
        if (y_goldencsc[i] != y[i]) error_count_check_cpu++;
    if (error_count_check_cpu != 0) printf("Check NO PASS! error_count_check_cpu= %d \n", error_count_check_cpu);
    else printf("Check FASTLOAD CPU PASS!\n");

    std::fill(y.begin(), y.end(), 0.0);
    char name[] = "dropin";
    FastLoad_spmv(name, matrixA, nnz, colA, rowA, sortx.data(), y.data(), y_goldencsr.data());

    // the reference's comparators (CSCSpMV.h: 1% check; cusparse_cuda.h: exact check)
    std::vector<double> yc(rowA, 0.0);
    const double ms_csc = csc_spmv_gpu_ms(rowA, colA, nnz, csccolptr.data(), cscrowidx.data(), cscval.data(),
                                          x.data(), yc.data(), 100);
    int bad_csc = ms_csc < 0;
    for (int i = 0; i < rowA && !bad_csc; i++)
        if (std::abs(y_goldencsr[i] - yc[i]) > 0.01 * std::abs(yc[i])) bad_csc++;
    if (!bad_csc) printf("BASIC CSC GPU PASS! (%f ms %4.2f GFlops)\n", ms_csc, 2.0 * nnz * 1.0e-6 / ms_csc);
    else printf("BASIC CSC check NO PASS! error_count_cuda = %d \n", bad_csc);
    std::vector<double> ys(rowA, 0.0);
    const double ms_cs = cusparse_spmv_gpu_ms(nnz, rowA, colA, csrrowptr.data(), csrcolidx.data(), csrval.data(),
                                              x.data(), ys.data(), 10);
    bool ok_cs = ms_cs >= 0;
    for (int i = 0; i < rowA && ok_cs; i++) ok_cs = ys[i] == y_goldencsr[i];
    if (ok_cs) printf("cuSPARSE test PASSED! (%f ms %4.2f GFlops)\n", ms_cs, 2.0 * nnz * 1.0e-6 / ms_cs);
    else printf("cuSPARSE test FAILED: wrong result\n");
    int exact = 0;
    for (int i = 0; i < rowA; i++) exact += y[i] == y_goldencsr[i];
    printf("exact %d of %d\n", exact, rowA);
    Tile_destroy(matrixA);
    free(matrixA);
    return (error_count_check == 0 && error_count_check_cpu == 0 && exact == rowA) ? 0 : 1;
}
