// ref_shim.cpp -- C entry points over the reference's own CPU path.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile (target `ref`) with the
// reference's src/ directory on the include path, so the functions below run
// the reference's unmodified code: mmio_allinone (src/auxiliary.h:65-232),
// csr2csc (src/coo2csc.h:11-72), col_sort (:75-129), formattransation
// (:132-312), tile_classification (:314-448) and FastLoad_cpu
// (src/FastLoad_CPU.h:2-46).  The output goes to oracle/_ref/ and is used to
// pin the C oracle and to produce the golden fixtures under tests/golden/.
// Arrays the reference allocates are copied into caller buffers and freed.
#include "coo2csc.h"
#include "FastLoad_CPU.h"

#include <cstdlib>
#include <cstring>

extern "C" {

// Reads a MatrixMarket file with the reference's reader.  First call with
// rowptr == nullptr returns the sizes; second call copies the CSR arrays.
int ref_mmio_read(const char *path, int *m, int *n, int *nnz, int *isSym,
                  int *rowptr, int *colidx, double *val)
{
    int *rp = nullptr, *ci = nullptr;
    double *v = nullptr;
    int rc = mmio_allinone(m, n, nnz, isSym, &rp, &ci, &v, const_cast<char *>(path));
    if (rc != 0) return rc;
    if (rowptr) {
        memcpy(rowptr, rp, sizeof(int) * (*m + 1));
        memcpy(colidx, ci, sizeof(int) * (*nnz));
        memcpy(val, v, sizeof(double) * (*nnz));
    }
    free(rp);
    free(ci);
    free(v);
    return 0;
}

void ref_csr2csc(int m, int n, int nnz, const int *rowptr, const int *colidx,
                 const double *val, int *cscptr, int *cscrow, double *cscval,
                 int *nnzpercol)
{
    int *r = nullptr, *p = nullptr, *c = nullptr;
    double *v = nullptr;
    csr2csc(nnz, m, n, const_cast<int *>(colidx), const_cast<int *>(rowptr),
            const_cast<double *>(val), &r, &p, &c, &v);
    memcpy(cscrow, r, sizeof(int) * nnz);
    memcpy(cscptr, p, sizeof(int) * (n + 1));
    memcpy(nnzpercol, c, sizeof(int) * n);
    memcpy(cscval, v, sizeof(double) * nnz);
    free(r);
    free(p);
    free(c);
    free(v);
}

// The reference CPU column sort (std::sort: tie order unspecified).
void ref_col_sort(int n, int nnz, const int *nnzpercol, const int *cscptr,
                  const int *cscrow, const double *cscval, const double *x,
                  int *sortrowidx_tmp, double *sortval_tmp, int *sortnnz,
                  double *sortx)
{
    col_sort(n, const_cast<int *>(nnzpercol), const_cast<int *>(cscptr),
             const_cast<int *>(cscrow), const_cast<double *>(cscval),
             sortrowidx_tmp, sortval_tmp, sortnnz, const_cast<double *>(x),
             sortx, nnz);
}

// Runs formattransation + tile_classification on caller-provided sorted
// arrays.  Returns the slide_matrix through a heap pointer that the caller
// reads with ref_layout_get and frees with ref_layout_free.
void *ref_layout_build(int m, int n, int nnz, const int *sortrowidx_tmp,
                       const double *sortval_tmp, const int *sortnnz)
{
    slide_matrix *mat = (slide_matrix *)calloc(1, sizeof(slide_matrix));
    formattransation(mat, const_cast<int *>(sortrowidx_tmp),
                     const_cast<double *>(sortval_tmp),
                     const_cast<int *>(sortnnz), nnz, m, n, 0);
    tile_classification(mat, nnz, m, n);
    return mat;
}

void ref_layout_sizes(void *h, int *tilenum, int *segsum)
{
    slide_matrix *mat = (slide_matrix *)h;
    *tilenum = mat->tilenum;
    *segsum = mat->segsum;
}

void ref_layout_get(void *h, int nnz, int *tile_ptr, int *tile_len,
                    int *tile_colidx, int *tile_tall, int *tile_format,
                    int *countrow, int *segmentoffset, int *sortrowindex,
                    int *sortrowidx, double *sortval)
{
    slide_matrix *mat = (slide_matrix *)h;
    int T = mat->tilenum, S = mat->segsum;
    memcpy(tile_ptr, mat->tile_ptr, sizeof(int) * (T + 1));
    memcpy(tile_len, mat->tile_len, sizeof(int) * T);
    memcpy(tile_colidx, mat->tile_colidx, sizeof(int) * T);
    memcpy(tile_tall, mat->tile_tall, sizeof(int) * T);
    memcpy(tile_format, mat->tile_format, sizeof(int) * T);
    memcpy(countrow, mat->countrow, sizeof(int) * (T + 1));
    memcpy(segmentoffset, mat->segmentoffset, sizeof(int) * (S + 1));
    memcpy(sortrowindex, mat->sortrowindex, sizeof(int) * nnz);
    memcpy(sortrowidx, mat->sortrowidx, sizeof(int) * nnz);
    memcpy(sortval, mat->sortval, sizeof(double) * nnz);
}

// FastLoad_cpu writes y += A x and prints a line when y differs from the
// golden it is given; the caller passes its own golden.
void ref_fastload_cpu(void *h, int nnz, int m, int n, const double *sortx,
                      double *y, const double *y_golden)
{
    FastLoad_cpu((slide_matrix *)h, nnz, m, n, const_cast<double *>(sortx), y,
                 const_cast<double *>(y_golden));
}

void ref_layout_free(void *h)
{
    slide_matrix *mat = (slide_matrix *)h;
    Tile_destroy(mat);
    free(mat);
}

}  // extern "C"
