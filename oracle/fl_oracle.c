/*
 * fl_oracle.c -- CPU oracle for the FastLoad CSC SpMV path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA library, never part of
 * the product path.  See fl_oracle.h for the contract and the parity pin.
 * Compiled with -ffp-contract=off so that x86 and Arm hosts round the
 * y[row] += val * x updates identically (no fused multiply-add).
 */
#include "fl_oracle.h"

#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Exclusive scan in place over len entries (src/auxiliary.h:29-44). */
static void excl_scan(int *a, long len)
{
    int run = 0;
    for (long i = 0; i < len; i++) {
        int v = a[i];
        a[i] = run;
        run += v;
    }
}

int fo_csr2csc(int m, int n, int nnz, const int *rowptr, const int *colidx,
               const double *val, int *cscptr, int *cscrow, double *cscval,
               int *nnzpercol)
{
    /* coo2csc.h:31-36: column counts. */
    memset(nnzpercol, 0, sizeof(int) * (size_t)n);
    for (int p = 0; p < nnz; p++) nnzpercol[colidx[p]]++;
    for (int j = 0; j < n; j++) cscptr[j] = nnzpercol[j];
    cscptr[n] = 0;
    excl_scan(cscptr, (long)n + 1);
    if (cscptr[n] != nnz) return -1;
    /* coo2csc.h:44-56: scatter rows in ascending order through a cursor per
     * column, which keeps rows ascending inside each column. */
    int *cursor = (int *)malloc(sizeof(int) * ((size_t)n + 1));
    if (!cursor) return -2;
    memcpy(cursor, cscptr, sizeof(int) * ((size_t)n + 1));
    for (int i = 0; i < m; i++) {
        for (int p = rowptr[i]; p < rowptr[i + 1]; p++) {
            int q = cursor[colidx[p]]++;
            cscrow[q] = i;
            cscval[q] = val[p];
        }
    }
    free(cursor);
    return 0;
}

int fo_col_sort(int n, const int *nnzpercol, const int *cscptr,
                const int *cscrow, const double *cscval, const double *x,
                int *perm, int *sortrowidx_tmp, double *sortval_tmp,
                int *sortnnz, double *sortx)
{
    /* Stable ascending order of columns by nonzero count: a counting sort
     * keyed on nnz per column keeps equal keys in ascending column id, the
     * order thrust::sort_by_key gives in ColSort_GPU.h:101. */
    int maxk = 0;
    for (int j = 0; j < n; j++)
        if (nnzpercol[j] > maxk) maxk = nnzpercol[j];
    int *bucket = (int *)calloc((size_t)maxk + 2, sizeof(int));
    if (!bucket) return -2;
    for (int j = 0; j < n; j++) bucket[nnzpercol[j]]++;
    excl_scan(bucket, (long)maxk + 2);
    for (int j = 0; j < n; j++) perm[bucket[nnzpercol[j]]++] = j;
    free(bucket);
    /* coo2csc.h:102-110 / ColSort_GPU.h:9-19: sorted x and counts. */
    for (int i = 0; i < n; i++) {
        sortx[i] = x[perm[i]];
        sortnnz[i] = nnzpercol[perm[i]];
    }
    /* coo2csc.h:113-128: concatenate the columns in sorted order. */
    long t = 0;
    for (int i = 0; i < n; i++) {
        int c = perm[i];
        for (int p = cscptr[c]; p < cscptr[c + 1]; p++, t++) {
            sortrowidx_tmp[t] = cscrow[p];
            sortval_tmp[t] = cscval[p];
        }
    }
    return 0;
}

/* Step k of the staircase: sorted column k starts a step when its count
 * exceeds the previous column's (coo2csc.h:153-186: exclusive_reduce, then
 * fortilecol/fortilennz/fortiletall). */
static int step_tall(const int *sortnnz, int k)
{
    return sortnnz[k] - (k ? sortnnz[k - 1] : 0);
}

int fo_count_tiles(int n, const int *sortnnz, int *h_count, int *tilenum)
{
    long long tiles = 0;
    int steps = 0;
    for (int k = 0; k < n; k++) {
        int tall = step_tall(sortnnz, k);
        if (tall != 0) {
            steps++;
            tiles += (long long)((n - k + 31) / 32) * tall; /* coo2csc.h:198-205 */
        }
    }
    *h_count = steps;
    if (tiles > 0x7fffffffLL) return -1;
    *tilenum = (int)tiles;
    return 0;
}

int fo_format_transform(int n, int nnz, const int *sortnnz,
                        const int *sortrowidx_tmp, const double *sortval_tmp,
                        int tilenum, int *tile_ptr, int *tile_len,
                        int *tile_colidx, int *tile_tall, int *sortrowidx,
                        double *sortval)
{
    int *colptr = (int *)malloc(sizeof(int) * ((size_t)n + 1));
    int *level = (int *)malloc(sizeof(int) * ((size_t)tilenum + 1));
    if (!colptr || !level) {
        free(colptr);
        free(level);
        return -2;
    }
    for (int k = 0; k < n; k++) colptr[k] = sortnnz[k];
    colptr[n] = 0;
    excl_scan(colptr, (long)n + 1); /* coo2csc.h:154 */

    /* coo2csc.h:229-250: tiles ordered by step, then 32-column chunk
     * (aligned to the step's first column), then level. */
    long t = 0;
    for (int k = 0; k < n; k++) {
        int tall = step_tall(sortnnz, k);
        if (tall == 0) continue;
        int base = k ? sortnnz[k - 1] : 0;
        int chunks = (n - k + 31) / 32;
        for (int j = 0; j < chunks; j++) {
            int len = (j == chunks - 1) ? n - k - (chunks - 1) * 32 : 32;
            for (int jx = 0; jx < tall; jx++, t++) {
                tile_len[t] = len;
                tile_colidx[t] = k + 32 * j;
                level[t] = base + jx;
            }
        }
    }
    if (t != tilenum) {
        free(colptr);
        free(level);
        return -1;
    }
    for (long i = 0; i < tilenum; i++) {
        tile_ptr[i] = tile_len[i];
        tile_tall[i] = 0; /* allocated and zeroed, never written: coo2csc.h:218-219 */
    }
    tile_ptr[tilenum] = 0;
    excl_scan(tile_ptr, (long)tilenum + 1); /* coo2csc.h:260 */
    if (tile_ptr[tilenum] != nnz) {
        free(colptr);
        free(level);
        return -1;
    }
    /* coo2csc.h:281-296: lane i of tile t holds the level-th nonzero of
     * sorted column tile_colidx[t] + i. */
    for (long i = 0; i < tilenum; i++) {
        for (int l = 0; l < tile_len[i]; l++) {
            int src = colptr[tile_colidx[i] + l] + level[i];
            int dst = tile_ptr[i] + l;
            sortval[dst] = sortval_tmp[src];
            sortrowidx[dst] = sortrowidx_tmp[src];
        }
    }
    free(colptr);
    free(level);
    return 0;
}

int fo_tile_classification(int nnz, int tilenum, const int *tile_ptr,
                           const int *tile_len, const int *sortrowidx,
                           int *tile_format, int *countrow,
                           int *segmentoffset, int *sortrowindex,
                           int *segsum)
{
    (void)nnz;
    /* coo2csc.h:362-381: runs of equal consecutive rows per tile, then an
     * exclusive scan gives each tile's first run index and segsum. */
    for (long i = 0; i < tilenum; i++) {
        int s = tile_ptr[i], len = tile_len[i], runs = 1;
        for (int j = s + 1; j < s + len; j++)
            if (sortrowidx[j] != sortrowidx[j - 1]) runs++;
        countrow[i] = runs;
        /* coo2csc.h:341-345 and 442-445: full tiles are format 1 (one run)
         * or 2 (several runs); partial tiles stay format 0. */
        tile_format[i] = (len == 32) ? (runs == 1 ? 1 : 2) : 0;
    }
    countrow[tilenum] = 0;
    excl_scan(countrow, (long)tilenum + 1);
    *segsum = countrow[tilenum];
    /* coo2csc.h:391-446: segmentoffset[r] = length of run r (with a zero
     * sentinel at segsum); sortrowindex marks each run head with its
     * length and is zero elsewhere. */
    for (long i = 0; i < tilenum; i++) {
        int s = tile_ptr[i], e = s + tile_len[i];
        int r = countrow[i];
        int head = s;
        for (int j = s + 1; j <= e; j++) {
            if (j == e || sortrowidx[j] != sortrowidx[head]) {
                segmentoffset[r++] = j - head;
                sortrowindex[head] = j - head;
                for (int q = head + 1; q < j; q++) sortrowindex[q] = 0;
                head = j;
            }
        }
    }
    segmentoffset[*segsum] = 0;
    return 0;
}

void fo_fastload_spmv(int tilenum, const int *tile_ptr, const int *tile_len,
                      const int *tile_colidx, const int *sortrowidx,
                      const double *sortval, const double *sortx, double *y)
{
    /* FastLoad_CPU.h:19-31. */
    for (int i = 0; i < tilenum; i++) {
        int start = tile_ptr[i], stop = tile_ptr[i + 1], len = tile_len[i];
        for (int j = start; j < stop; j++)
            y[sortrowidx[j]] += sortval[j] * sortx[tile_colidx[i] + (j - start) % len];
    }
}

int fo_fastload_spmv_omp(int tilenum, const int *tile_ptr,
                         const int *tile_len, const int *tile_colidx,
                         const int *sortrowidx, const double *sortval,
                         const double *sortx, double *y, int nthreads)
{
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
    int used = 1;
#pragma omp parallel num_threads(nthreads)
    {
#pragma omp single
        used = omp_get_num_threads();
#pragma omp for schedule(dynamic, 256)
        for (int i = 0; i < tilenum; i++) {
            int start = tile_ptr[i], stop = tile_ptr[i + 1], len = tile_len[i];
            for (int j = start; j < stop; j++) {
                double v = sortval[j] * sortx[tile_colidx[i] + (j - start) % len];
#pragma omp atomic
                y[sortrowidx[j]] += v;
            }
        }
    }
    return used;
#else
    (void)nthreads;
    fo_fastload_spmv(tilenum, tile_ptr, tile_len, tile_colidx, sortrowidx,
                     sortval, sortx, y);
    return 1;
#endif
}

void fo_csc_spmv(int n, const int *cscptr, const int *cscrow,
                 const double *cscval, const double *x, double *y)
{
    for (int c = 0; c < n; c++)
        for (int p = cscptr[c]; p < cscptr[c + 1]; p++)
            y[cscrow[p]] += cscval[p] * x[c];
}

void fo_csr_spmv(int m, const int *rowptr, const int *colidx,
                 const double *val, const double *x, double *y)
{
    for (int i = 0; i < m; i++) {
        double s = 0;
        for (int p = rowptr[i]; p < rowptr[i + 1]; p++) s += val[p] * x[colidx[p]];
        y[i] = s;
    }
}

void fo_csc_spmv_dd(int m, int n, int k, const int *cscptr,
                    const int *cscrow, const double *cscval, const double *x,
                    double *y)
{
    size_t cnt = (size_t)m * (size_t)k;
    double *lo = (double *)calloc(cnt ? cnt : 1, sizeof(double));
    for (size_t i = 0; i < cnt; i++) y[i] = 0.0;
    for (int c = 0; c < n; c++) {
        for (int p = cscptr[c]; p < cscptr[c + 1]; p++) {
            size_t r0 = (size_t)cscrow[p] * (size_t)k;
            for (int r = 0; r < k; r++) {
                double a = cscval[p], b = x[(size_t)c * k + r];
                double prod = a * b;
                double perr = fma(a, b, -prod); /* exact product error */
                double s = y[r0 + r] + prod;    /* Knuth TwoSum */
                double bb = s - y[r0 + r];
                double serr = (y[r0 + r] - (s - bb)) + (prod - bb);
                y[r0 + r] = s;
                lo[r0 + r] += serr + perr;
            }
        }
    }
    for (size_t i = 0; i < cnt; i++) y[i] += lo[i];
    free(lo);
}

/* ------------------------------------------------------- MatrixMarket -- */
/* Banner: five fields, the first starting with %%MatrixMarket, the others
 * compared in lower case (src/mmio.h:172-259).  field: 'R','I','P','C';
 * storage: 'G','S','H','K'. */
static int mm_banner(FILE *f, char *field, char *storage)
{
    char line[1025], b[1025], obj[1025], fmt[1025], typ[1025], sto[1025];
    if (!fgets(line, sizeof line, f)) return -2;
    if (sscanf(line, "%s %s %s %s %s", b, obj, fmt, typ, sto) != 5) return -2;
    for (char *p = obj; *p; p++) *p = (char)tolower((unsigned char)*p);
    for (char *p = fmt; *p; p++) *p = (char)tolower((unsigned char)*p);
    for (char *p = typ; *p; p++) *p = (char)tolower((unsigned char)*p);
    for (char *p = sto; *p; p++) *p = (char)tolower((unsigned char)*p);
    if (strncmp(b, "%%MatrixMarket", 14) != 0) return -2;
    if (strcmp(obj, "matrix") != 0 || strcmp(fmt, "coordinate") != 0) return -2;
    if (!strcmp(typ, "real")) *field = 'R';
    else if (!strcmp(typ, "integer")) *field = 'I';
    else if (!strcmp(typ, "pattern")) *field = 'P';
    else if (!strcmp(typ, "complex")) *field = 'C';
    else return -2;
    if (!strcmp(sto, "general")) *storage = 'G';
    else if (!strcmp(sto, "symmetric")) *storage = 'S';
    else if (!strcmp(sto, "hermitian")) *storage = 'H';
    else if (!strcmp(sto, "skew-symmetric")) *storage = 'K';
    else return -2;
    return 0;
}

/* Size line after the comment lines (src/mmio.h:142-170). */
static int mm_size(FILE *f, int *m, int *n, int *nz)
{
    char line[1025];
    do {
        if (!fgets(line, sizeof line, f)) return -4;
    } while (line[0] == '%');
    if (sscanf(line, "%d %d %d", m, n, nz) == 3) return 0;
    /* a blank line: the sizes are the next three tokens (a token that is not
     * an integer is an error; the reference would spin on it) */
    return fscanf(f, "%d %d %d", m, n, nz) == 3 ? 0 : -4;
}

int fo_mmio_read(const char *path, int *m, int *n, int *nnz, int *is_symmetric,
                 int *rowptr, int *colidx, double *val)
{
    FILE *f = fopen(path, "r");
    if (!f) return -1;
    char field = 0, storage = 0;
    int rc = mm_banner(f, &field, &storage);
    int M = 0, N = 0, NZ = 0;
    if (!rc) rc = mm_size(f, &M, &N, &NZ);
    if (rc) {
        fclose(f);
        return rc;
    }
    const int sym = storage == 'S' || storage == 'H';
    if (sym && M != N) { /* mirrored entries would fall outside the matrix */
        fclose(f);
        return -5;
    }
    int *ri = (int *)malloc(sizeof(int) * (NZ ? NZ : 1));
    int *ci = (int *)malloc(sizeof(int) * (NZ ? NZ : 1));
    double *vv = (double *)malloc(sizeof(double) * (NZ ? NZ : 1));
    int *cnt = (int *)calloc((size_t)M + 1, sizeof(int));
    rc = (ri && ci && vv && cnt) ? 0 : -5;
    for (int i = 0; i < NZ && !rc; i++) {
        int r, c, iv, got;
        double v = 1.0, im;
        if (field == 'R') got = fscanf(f, "%d %d %lg", &r, &c, &v) == 3;
        else if (field == 'C') got = fscanf(f, "%d %d %lg %lg", &r, &c, &v, &im) == 4;
        else if (field == 'I') {
            got = fscanf(f, "%d %d %d", &r, &c, &iv) == 3;
            v = iv;
        } else got = fscanf(f, "%d %d", &r, &c) == 2;
        if (!got || r < 1 || r > M || c < 1 || c > N) {
            rc = -5;
            break;
        }
        ri[i] = r - 1;
        ci[i] = c - 1;
        vv[i] = v;
        cnt[r - 1]++;
        if (sym && r != c) cnt[c - 1]++;
    }
    fclose(f);
    if (!rc) {
        excl_scan(cnt, (long)M + 1);
        *m = M;
        *n = N;
        *nnz = cnt[M];
        *is_symmetric = sym;
        if (rowptr) {
            memcpy(rowptr, cnt, sizeof(int) * ((size_t)M + 1));
            /* fill rows in file order; a mirrored entry follows its original */
            for (int i = 0; i < NZ; i++) {
                int p = cnt[ri[i]]++;
                colidx[p] = ci[i];
                val[p] = vv[i];
                if (sym && ri[i] != ci[i]) {
                    p = cnt[ci[i]]++;
                    colidx[p] = ri[i];
                    val[p] = vv[i];
                }
            }
        }
    }
    free(ri);
    free(ci);
    free(vv);
    free(cnt);
    return rc;
}
