/*
 * ent_oracle.h -- CPU oracle for the entropical density hot path.
 *
 * TEST INFRASTRUCTURE ONLY. Nothing in the product (the CUDA library, its
 * C ABI or the Python host mirror) links, loads or calls this code; only the
 * tests, the smoke check and the CPU-baseline leg of the benchmark do, and
 * only as the checker. Every function restates one piece of the reference
 * (lettis/entropical) on the CPU, citing the reference file:line it follows,
 * or is the FP64 brute force the reference's float results are judged by.
 *
 * Parity pinning: the reference ships no tests or golden vectors. These
 * restatements are pinned against the reference's own OpenMP sources compiled
 * from source (oracle/_ref, built by oracle/Makefile), and golden fixtures
 * generated from that build are committed under tests/golden/. Boost is not
 * available, so the Kahan-sum and lazy-variance features the reference takes
 * from Boost.Accumulators are restated from their textbook definitions
 * (parity unpinned at that one boundary).
 *
 * Layout conventions follow the reference: coordinates are column-major
 * float32, column j of an n-row buffer at sel[j*n + i].
 */
#ifndef ENT_ORACLE_H
#define ENT_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* FP64 brute-force product-Epanechnikov density at selected targets:
 *   out[t] = (1/norm) * sum_s prod_j 0.75*(1-u_j^2)/h_j * [u_j^2 <= 1],
 *   u_j = (x_tj - x_sj)/h_j, all in double; compact support makes the
 *   window on dimension 0 exact. (densities_omp.cpp:19-26, :67-159) */
int orc_density_fp64_at(const float* sel, size_t n, int d, const double* h,
                        double norm, const uint32_t* targets, size_t n_targets,
                        double* out);
int orc_density_fp64(const float* sel, size_t n, int d, const double* h,
                     double norm, double* out);
/* Number of ordered pairs (i, k) with |x_ij - x_kj| <= h_j for every j. */
uint64_t orc_support_count_fp64(const float* sel, size_t n, int d,
                                const double* h);

/* Float restatement of the reference OpenMP density, operation for operation:
 * dim-1 sort (tools.hxx:113-150), boxes() windows (densities_omp.cpp:33-65),
 * float accumulation of epanechnikov() products (:19-26, :67-159), then /n. */
int orc_density_ref_f32(const float* sel, size_t n, int d, const float* h,
                        float* out);
/* Same result with the reference's linear window scans (its O(n^2) cost);
 * used only to time the CPU baseline. */
int orc_density_ref_f32_linear(const float* sel, size_t n, int d,
                               const float* h, float* out);

/* boxes() window bounds (densities_omp.cpp:33-65) for every point of a column
 * (original order) against the sorted column: lo = first k with
 * x - s[k] < h, hi = last k with s[k] - x < h (strict float compares). */
void orc_boxes(const float* col, size_t n, float h, uint64_t* lo, uint64_t* hi);

/* Transs::BoxedSearch::Boxes (boxedsearch.cpp:15-62) with its undefined
 * cases defined: the maximum starts at -FLT_MAX, a box index equal to the box
 * count is clamped to the last box, and a zero-width range gives one box.
 * Returns the box count; fills each state's box and neighbour-list size. */
uint64_t orc_boxedsearch(const float* col, size_t n, float box_size,
                         uint64_t* box_of_state, uint64_t* n_neighbors);

/* epa_convolution (densities_omp.cpp:235-277), float, Kahan per row over all
 * n entries (zeros included) and across rows. O(n^2): small n only. */
float orc_epa_conv_ref(const float* sorted, size_t n, float h);
/* Exact FP64 value of the same convolution sum. */
double orc_epa_conv_fp64(const float* sorted, size_t n, double h);

/* Hestimate::Thumb::Kernel (hestimate.cpp:19-30): n^(-1/7) * sqrt(lazy
 * variance accumulated in float). */
float orc_thumb_ref(const float* col, size_t n);
/* AmiseMin::_amise (hestimate.cpp:41-53) given the convolution value. */
float orc_amise_from_conv(float conv, float h, size_t n);
/* AmiseMin::operator() (hestimate.cpp:88-104) with the interval search
 * (:55-86). exact_conv=1 uses orc_epa_conv_ref (O(n^2)), 0 the FP64 value
 * rounded to float. n_conv (optional) receives the number of convolutions. */
float orc_hestimate_amise(const float* col, size_t n, int exact_conv,
                          int* n_conv);

/* XTC trajectories (xtc_oracle.c): the reading side of CoordsFile::
 * XtcHandler (coords_file/coords_file.cpp:90-110, xdrfile_xtc.c:83-95,
 * xdrfile.c:761-961). orc_xtc_shape: frames up to the first that does not
 * parse, and the atom count (0 ok, -1 unreadable, -2 no frame).
 * orc_read_xtc: frames [f0, f1) into out[(3a + c) * n_out_rows + (f - f0)]
 * (x, y, z of atom a: columns 3a, 3a+1, 3a+2); returns the frames read, or
 * -1 (unreadable) / -2 (malformed compressed frame). */
int orc_xtc_shape(const char* path, size_t* n_frames, size_t* n_atoms);
long orc_read_xtc(const char* path, size_t f0, size_t f1, float* out, size_t n_out_rows);

#ifdef __cplusplus
}
#endif
#endif
