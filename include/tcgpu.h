/* tcgpu.h -- C ABI of the GB300 (sm_103a) engine for TreeCorr's 2-point correlation
 * hot path: ball-tree build, dual-tree traversal with the bin_slop accept/split rule, and
 * the per-pair NN / KK / GG accumulation with Log binning on Flat, ThreeD and Sphere
 * coordinates (Euclidean and Arc metrics).
 *
 * Each entry point replaces one call of the reference's native module `_treecorr`
 * (TreeCorr's pybind11 layer); the reference file:line is given beside it.  Arguments keep
 * the reference's names, order and meaning.  Differences at the boundary:
 *   - plain pointers and sizes instead of numpy buffers; an absent optional array
 *     (z, wpos, an unused xi) is NULL instead of an empty array;
 *   - every call returns a status code (TC_OK == 0) instead of printing an Assert and
 *     continuing; tc_last_error() gives the message of the calling thread's last failure.
 *
 * Ownership: a field owns its device copy of the catalog and its tree (tc_field_free).
 * A corr object aliases the caller's output arrays, exactly like BuildCorr2
 * (src/Corr2.cpp:842-864): they must outlive it, and every process call only ADDS into
 * them (clearing them is the caller's job, as in treecorr/corr2base.py:1296-1306).
 *
 * All work runs on the current CUDA device, on the library's own stream; calls return
 * after the results are in the caller's arrays.  One corr object must not be used from
 * two threads at once (its outputs are aliased), as in the reference.
 */
#ifndef TCGPU_H
#define TCGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define TC_OK               0
#define TC_ERR_ARG          1   /* invalid argument (sizes, enums, NULL where required) */
#define TC_ERR_CUDA         2   /* a CUDA runtime call failed */
#define TC_ERR_UNSUPPORTED  3   /* combination outside the GPU path (e.g. Rperp metric) */
#define TC_ERR_DEVICE       4   /* a kernel reported an error through its status word */
#define TC_ERR_NOMEM        5   /* device allocation failed */

/* Enumerations: same numeric values as the reference's enums. */
/* Coord, include/Position.h:24 */
#define TC_FLAT    1
#define TC_THREED  2
#define TC_SPHERE  3
/* Metric, include/Metric.h:29 */
#define TC_EUCLIDEAN 1
#define TC_RPERP     2
#define TC_RLENS     3
#define TC_ARC       4
#define TC_OLDRPERP  5
#define TC_PERIODIC  6
/* SplitMethod, include/Cell.h:26 */
#define TC_MIDDLE 0
#define TC_MEDIAN 1
#define TC_MEAN   2
#define TC_RANDOM 3
/* BinType, include/BinType.h:36 */
#define TC_LOG          0
#define TC_LINEAR       1
#define TC_TWOD         2
#define TC_LOGRUV       3
#define TC_LOGSAS       4
#define TC_LOGMULTIPOLE 5
/* Data kinds of a field (DataType, include/Cell.h:37; this ABI numbers them N, K, G, Z,
 * V, T, Q = 0..6, the reference N, K, Z, V, G, T, Q = 0..6 -- Python passes classes, not
 * numbers, so only the names must agree). */
#define TC_NDATA 0   /* counts */
#define TC_KDATA 1   /* scalar */
#define TC_GDATA 2   /* spin-2 complex (shear) */
#define TC_ZDATA 3   /* spin-0 complex */
#define TC_VDATA 4   /* spin-1 complex (vector) */
#define TC_TDATA 5   /* spin-3 complex */
#define TC_QDATA 6   /* spin-4 complex */

typedef struct tc_field tc_field;
typedef struct tc_corr2 tc_corr2;
typedef struct tc_corr3 tc_corr3;

/* Counters of the last process call (no reference counterpart; the reference has none). */
typedef struct tc_stats {
    int64_t cell_pairs;      /* cell pairs evaluated by the traversal */
    int64_t accepted;        /* cell pairs accumulated (directProcess11 calls) */
    int64_t escalated;       /* decisions re-done in FP64 near a threshold */
    int64_t launches;        /* traversal kernel launches */
    double  build_ms;        /* device time of the tree builds done by this call */
    double  traverse_ms;     /* device time of the traversal + reduction */
    int64_t learned;         /* cell pairs accepted by the learned criterion (of accepted) */
    int64_t tiles;           /* leaf-pair tiles of the exact mode (angle_slop 0 or brute) */
    int64_t tile_pairs;      /* leaf pairs evaluated in tiles (accepted ones are in accepted) */
    int64_t tile_escalated;  /* tile leaf pairs decided again in FP64 near a bin edge */
    double  expand_ms;       /* device time of the expansion launches (k_expand) */
    double  tiles_ms;        /* device time of the tile launches (k_tiles) */
} tc_stats;

/* Field construction: replaces BuildNField / BuildKField / BuildZField / BuildVField /
 * BuildGField / BuildTField / BuildQField for C = Flat, Sphere, ThreeD (src/Field.cpp:430-560,
 * pybind11 constructors at 683-689), i.e. Field<D,C>::Field (src/Field.cpp:163-204).
 * Host arrays of length n:
 *   x, y: positions; z: NULL for Flat; d1 = k (K) or the real part (Z, V, G, T, Q),
 *   d2 = the imaginary part;
 *   w: weights; wpos: NULL means "use w" (src/Field.cpp:146-152).
 * The data are copied to the device here; the tree is built on the first call that needs
 * it (tc_field_ntop or a process call), like the reference's lazy BuildCells.  A non-zero
 * seed reseeds the random stream of the k-means initialisations, as BaseField's constructor
 * does (src/Field.cpp:160). */
int tc_field_create(int dkind, int coords,
                    const double* x, const double* y, const double* z,
                    const double* d1, const double* d2,
                    const double* w, const double* wpos, int64_t n,
                    double min_size, double max_size, int split_method, int64_t seed,
                    int brute, int min_top, int max_top, tc_field** out);

/* Same as tc_field_create, but the arrays are DEVICE pointers already resident on the
 * current device (no counterpart in the reference: it is the device-resident form of the
 * same constructor, for callers whose catalog already lives in HBM). */
int tc_field_create_device(int dkind, int coords,
                           const double* x, const double* y, const double* z,
                           const double* d1, const double* d2,
                           const double* w, const double* wpos, int64_t n,
                           double min_size, double max_size, int split_method, int64_t seed,
                           int brute, int min_top, int max_top, tc_field** out);

/* ~BaseField, src/Field.cpp:279-285. */
void tc_field_free(tc_field* f);

/* BaseField::getNObj, include/Field.h:52. */
int64_t tc_field_nobj(const tc_field* f);
/* BaseField::getSize, include/Field.h:55 (sqrt of the overall size^2). */
double tc_field_size(const tc_field* f);
/* BaseField::getNTopLevel, include/Field.h:56: builds the tree if needed; < 0 on error. */
int64_t tc_field_ntop(tc_field* f);
/* Overall centre (x,y,z) as in Field::Field, src/Field.cpp:198-203. */
int tc_field_center(const tc_field* f, double* xyz3);

/* Canonical depth-first dump of the tree (tops in order, left child before right) for
 * parity tests against the oracle: per cell its centre (xyz, 3 doubles), size, w, and
 * payload (4 floats), count and first point index in tree order (2 int64), and depth.
 * Returns the number of cells (writes at most cap of them), < 0 on error.  No reference
 * counterpart (BaseCell::WriteTree, src/Cell.cpp:703-710, is the closest). */
int64_t tc_field_dump(tc_field* f, double* xyz, float* size_w_d, int64_t* n_start,
                      int32_t* depth, int64_t cap);

/* k-means patches on the field's tree: the BaseField methods bound at
 * src/Field.cpp:630-634 (implemented in src/KMeans.cpp:743-849).  centers holds npatch
 * rows of 2 (Flat) or 3 (ThreeD, Sphere; unit vectors) doubles in host memory.  The
 * initialisations draw from the C library's rand() stream like the reference's urand()
 * (a non-zero seed reseeds it).  npatch is limited to 5000 on the GPU path. */
int tc_kmeans_init_tree(tc_field* f, double* centers, int npatch, int64_t seed);   /* KMeansInitTree */
int tc_kmeans_init_rand(tc_field* f, double* centers, int npatch, int64_t seed);   /* KMeansInitRand */
int tc_kmeans_init_kmpp(tc_field* f, double* centers, int npatch, int64_t seed);   /* KMeansInitKMPP */
/* KMeansRun (src/KMeans.cpp:773-833): refines centers in place. */
int tc_kmeans_run(tc_field* f, double* centers, int npatch, int max_iter, double tol, int alt);
/* KMeansAssign (src/KMeans.cpp:835-849): patches[i] for every point i of the field
 * (n must equal tc_field_nobj). */
int tc_kmeans_assign(tc_field* f, const double* centers, int npatch, int64_t* patches,
                     int64_t n);
/* Iterations run by the last tc_kmeans_run on this field (no reference counterpart). */
int tc_kmeans_iterations(const tc_field* f);

/* QuickAssign (src/KMeans.cpp:890-942, bound at src/Field.cpp:700): the nearest centre of
 * every point; z == NULL selects the 2-d form (centers npatch x 2). */
int tc_quick_assign(const double* centers, int npatch, const double* x, const double* y,
                    const double* z, int64_t n, int64_t* patches);
/* SelectPatch (src/KMeans.cpp:944-1011, bound at src/Field.cpp:701): use[i] = 1 when patch
 * is the nearest centre of point i (no other centre strictly closer), else 0. */
int tc_select_patch(int patch, const double* centers, int npatch, const double* x,
                    const double* y, const double* z, int64_t n, int64_t* use);
/* The same two with device pointers for x, y, z and the output (no host copies). */
int tc_quick_assign_device(const double* centers, int npatch, const double* x,
                           const double* y, const double* z, int64_t n, int64_t* patches);
int tc_select_patch_device(int patch, const double* centers, int npatch, const double* x,
                           const double* y, const double* z, int64_t n, int64_t* use);

/* Corr construction: replaces BuildCorr2 (src/Corr2.cpp:842-864) for the 18 classes of
 * src/Corr2.cpp:1204-1232: NN, NK, KK, and NX, KX, XX for X in Z, V, G, T, Q (d1 <= d2 as
 * there).  xi arrays used: none (NN); xi0 (NK, KK); xi0, xi1 = real, imaginary (NX, KX;
 * for NG and KG the tangential sign of DirectHelper<2>, src/Corr2.cpp:424-443); xi0..xi3 =
 * xip, xip_im, xim, xim_im (XX); the others may be NULL.  Only
 * bin_type == TC_LOG is on the GPU path; minrpar/maxrpar/xp/yp/zp are accepted and
 * must be the defaults (no r_parallel cut, no period). */
int tc_corr2_create(int d1, int d2, int bin_type, double minsep, double maxsep, int nbins,
                    double binsize, double b, double a,
                    double minrpar, double maxrpar, double xp, double yp, double zp,
                    double* xi0, double* xi1, double* xi2, double* xi3,
                    double* meanr, double* meanlogr, double* weight, double* npairs,
                    tc_corr2** out);

void tc_corr2_free(tc_corr2* c);

/* BaseCorr2.processAuto -> ProcessAuto (src/Corr2.cpp:913-929) ->
 * BaseCorr2::process(field) (src/Corr2.cpp:146-205).  quick == corr_only. */
int tc_corr2_process_auto(tc_corr2* c, tc_field* f, int dots, int quick, int metric);

/* BaseCorr2.processCross -> ProcessCross (src/Corr2.cpp:978-993) ->
 * BaseCorr2::process(field1, field2) (src/Corr2.cpp:207-288). */
int tc_corr2_process_cross(tc_corr2* c, tc_field* f1, tc_field* f2, int dots, int quick,
                           int metric);

/* The auto-correlation of tc_corr2_process_auto, for callers that cannot let this library
 * allocate GPU memory during the call: a process whose device memory is all handed out by
 * its own memory pool (so a cudaMalloc here would fail or evict the pool's cache), or a
 * latency-critical pipeline that must not take the device-wide synchronisation that
 * cudaMalloc and cudaFree can cause.  No reference counterpart: the reference runs on the
 * CPU and allocates per call.
 *
 * Nothing is allocated: the traversal's work lists and partial sums live in one fixed
 * device array of about 52 MiB that is part of this library (every GPU that loads the
 * library holds it until the process exits).  Limits: nbins <= 64, at most 1024 warps, and
 * work lists of the fixed size; a traversal that needs more space fails with
 * TC_ERR_DEVICE and a clear message (tc_corr2_process_auto has no such limit).  Only the
 * bin_slop criterion runs: a corr with the learned criterion set (tc_corr2_set_learned) is
 * refused with TC_ERR_ARG.  The field must already be built (call tc_field_ntop once
 * beforehand: building the tree allocates).  The first call on a device looks up the
 * array's device address (set-up, once per device, with that device current).  The
 * environment variable TCGPU_NOALLOC_SPILL_CAP (items) shortens the spill list, so that
 * tests reach the overflow path on small catalogs.  All calls share the array, which keeps the last
 * call's contents (each call clears what must start at zero): calls that overlap on the GPU
 * (from several host threads, or processes sharing a context) race and must be serialised
 * by the caller.  Results are added into the corr's output arrays as usual; in the stats,
 * traverse_ms stays 0. */
int tc_corr2_process_auto_noalloc(tc_corr2* c, tc_field* f, int quick, int metric);

/* Tuning of the 2-point path (no reference counterpart: the reference's OpenMP loop has no
 * such knobs).  tile_leaf: the most points per side of a leaf-pair tile of the exact mode
 * (8..64; 0 = the default 48); chunk: work items per expansion launch, the depth of the
 * breadth-first queue (2^16..2^26; 0 = the default: the smallest power of two at least
 * twice the points, between 2^16 and 2^25; 2^24 at most for the patch batch).  Neither
 * changes which pairs land in which bins; the sums agree to FP32 rounding (bit for bit
 * between runs with equal settings). */
int tc_corr2_set_tuning(tc_corr2* c, int tile_leaf, int64_t chunk);

/* The autotuner: times this correlation of f1 (and f2, NULL for an auto-correlation) on its
 * first frac of top-level cell pairs for tile leaf sizes 24..64 (exact mode only), then for
 * expansion chunks down to 1/8 of the default, keeps the fastest in c (as
 * tc_corr2_set_tuning) and in a per-process cache keyed by the classes, coordinates, metric,
 * binning, slops, brute flags and catalog sizes (to a factor of 2), so a later call with the
 * same key returns at once.  The corr's output arrays are not touched.  Outputs: the chosen
 * values (0 = default) and the best sample's device time in ms (0 from the cache).  No
 * reference counterpart. */
int tc_corr2_autotune(tc_corr2* c, tc_field* f1, tc_field* f2, int metric, double frac,
                      int* tile_leaf, int64_t* chunk, double* ms);

/* BaseCorr2.triviallyZero -> TriviallyZero (src/Corr2.cpp:1107-1128): 1 if no pair of
 * the two patches (centre + size) can fall in range.  Result in *out. */
int tc_corr2_trivially_zero(tc_corr2* c, int metric, int coords,
                            double x1, double y1, double z1, double s1,
                            double x2, double y2, double z2, double s2, int* out);

/* Counters of the last process call on c. */
int tc_corr2_stats(const tc_corr2* c, tc_stats* out);

/* 3-point correlation with LogMultipole binning: replaces BuildCorr3
 * (src/Corr3.cpp:3599-3645) for the 21 classes of the reference's module: N, K or G
 * (TC_NDATA, TC_KDATA, TC_GDATA) at each vertex, not all three different (pybind11 at
 * src/Corr3.cpp:4207-4262).  Arguments as the reference's (nubins = max_n; the u/v
 * arguments are unused by LogMultipole).  Every output has nbins*nbins*(2*max_n+1)
 * entries; the zeta arrays are those of the class's ZetaData (include/Corr3.h:581-720):
 * gam0r..gam3i in zeta0..7 with three G's, gam0r, gam0i, gam1r, gam1i in zeta0..3 with two,
 * zeta (real, imaginary) in zeta0, zeta1 with one or none, unused for NNN.  A class whose
 * vertices 2 and 3 differ runs through tc_corr3_process_cross21 / _cross only.
 * meand1, meanlogd1, meanu and meanv are accepted and left untouched, as the reference's
 * multipole code leaves them. */
int tc_corr3_create(int d1, int d2, int d3, int bin_type, double minsep, double maxsep,
                    int nbins, double binsize, double b, double a, double minu, double maxu,
                    int nubins, double ubinsize, double bu, double minv, double maxv,
                    int nvbins, double vbinsize, double bv, double minrpar, double maxrpar,
                    double xp, double yp, double zp, double* zeta0, double* zeta1,
                    double* zeta2, double* zeta3, double* zeta4, double* zeta5, double* zeta6,
                    double* zeta7, double* meand1, double* meanlogd1, double* meand2,
                    double* meanlogd2, double* meand3, double* meanlogd3, double* meanu,
                    double* meanv, double* weight, double* weight_im, double* ntri,
                    tc_corr3** out);

void tc_corr3_free(tc_corr3* c);

/* BaseCorr3.processAuto -> ProcessAutoc -> BaseCorr3::multipole (src/Corr3.cpp:3654-3669,
 * 1124-1175): the G_n / Gamma_n multipole accumulation over one G field. */
int tc_corr3_process_auto(tc_corr3* c, tc_field* f, int dots, int quick, int metric);

/* BaseCorr3.processCross12 -> ProcessCross12c (src/Corr3.cpp:4199, 3730-3768): one vertex
 * from f1, two from f2.  ordered = 1 runs multipole(field1, field2) (1177-1237); ordered = 0
 * adds the three-field multipole(field2, field1, field2, 1) first, as the reference does. */
int tc_corr3_process_cross12(tc_corr3* c, tc_field* f1, tc_field* f2, int ordered, int dots,
                             int quick, int metric);

/* BaseCorr3.processCross21 -> ProcessCross21c (src/Corr3.cpp:4200, 3831-3868): two vertices
 * from f1, one from f2, through the three-field multipole (1239-1305): ordered = 3 runs
 * multipole(f1, f1, f2, 4); ordered = 0 the three placements with ordered 1. */
int tc_corr3_process_cross21(tc_corr3* c, tc_field* f1, tc_field* f2, int ordered, int dots,
                             int quick, int metric);

/* BaseCorr3.processCross -> ProcessCrossc (src/Corr3.cpp:4201, 3938-3976): one vertex from
 * each field through the three-field multipole, with the reference's placements for
 * ordered = 0 .. 4.  Vertex 2's and 3's fields must share a data kind (d2 = d3). */
int tc_corr3_process_cross(tc_corr3* c, tc_field* f1, tc_field* f2, tc_field* f3,
                           int ordered, int dots, int quick, int metric);

/* Device time of the last tc_corr3_process_* call in ms, summed over its multipoles (no
 * reference counterpart). */
double tc_corr3_last_ms(const tc_corr3* c);

/* Counters of the last tc_corr3_process_auto call (no reference counterpart):
 * out[0] vertex records contracted in batches, out[1] records contracted in place because
 * the record buffer was full, out[2] finish/contract waves.  Returns TC_OK. */
int tc_corr3_stats(const tc_corr3* c, int64_t out[3]);

/* Patches: every patch-pair correlation of npatch patch fields in one expansion (replaces
 * the Python loop over patch pairs, treecorr/corr2base.py:929-950, and its processAuto /
 * processCross calls).  Pairs (i, j), i <= j, whose fields can overlap (triviallyZero,
 * src/Corr2.cpp:1107-1128) are processed; pair_i / pair_j receive them and results receives
 * per pair 8 arrays of nbins doubles: weight, meanr, meanlogr, xi0, xi1, xi2, xi3, npairs
 * (raw sums, as in the reference's results[(i, j)] before _finalize).  The corr's own
 * output arrays are not touched. */
int tc_corr2_process_patches(tc_corr2* corr, tc_field* const* fields, int npatch, int metric,
                             int quick, int max_pairs, int32_t* pair_i, int32_t* pair_j,
                             double* results, int* npairs_out);

/* Jackknife design matrix and covariance on the device from per-pair results (layout of
 * tc_corr2_process_patches): row l sums the pairs with the reference's weights
 * (JackknifePairIterator, corr2base.py:1787-1817; cross_patch_weight 0 simple, 1 mean,
 * 2 match), divides by the weight (_finalize) and takes the statistic (GG: xip, xim;
 * KK: xi); cov = (1 - 1/npatch) sum_l (v_l - mean)(v_l - mean)^T (_cov_jackknife,
 * corr2base.py:2432-2445).  v_out: npatch x nstat*nbins, cov_out: (nstat*nbins)^2. */
int tc_jackknife_cov(const double* results, const int32_t* pair_i, const int32_t* pair_j,
                     int npair, int npatch, int nbins, int dkind, int cross_patch_weight,
                     double* v_out, double* cov_out);

/* GenerateXYZ (src/KMeans.cpp:1013-1050, pybind11 at src/Field.cpp:700-702; caller
 * treecorr/catalog.py:1609-1622): x = cos(dec) cos(ra), y = cos(dec) sin(ra), z = sin(dec),
 * each times r[i] when r is not NULL.  Host arrays of length n (copied to the device and
 * back), or device arrays for tc_generate_xyz_device. */
int tc_generate_xyz(double* x, double* y, double* z, const double* ra, const double* dec,
                    const double* r, int64_t n);
int tc_generate_xyz_device(double* x, double* y, double* z, const double* ra,
                           const double* dec, const double* r, int64_t n);

/* Catalog ingestion: the column work of Catalog._finish_input (treecorr/catalog.py:
 * 1343-1487) on the GPU.  In order: flag -> weight (1393-1404: w = 0, and wpos = 0 when given,
 * where (flag & ignore_flag) != 0; the Python layer's ignore_flag is ~ok_flag unless given);
 * checkForNaN (1406-1425, 1684-1704) on the ncols columns in the given order, then on w,
 * then on wpos (a NaN row gets w = 0 and the NaN becomes 0); wpos == 0 -> w = 0 (1433-1450);
 * sumw (1452-1462); removal of the rows with wpos == 0 (w == 0 without wpos) unless
 * keep_zero_weight, when the weights are non-trivial (1464-1468, Catalog.select).  The
 * weights are non-trivial when w_given, flag != NULL, a NaN was found or some wpos is 0;
 * otherwise w is filled with 1 and sumw = n.  The columns (positions: x, y, z or ra, dec,
 * r; values: k, g1, g2, ...) are changed in place; removed rows are dropped keeping the
 * order, info->nkeep rows remain.  w: length n (the caller's weights when w_given, else any
 * buffer, filled here); wpos, flag: NULL when absent.  sumw == 0 with non-trivial weights
 * is TC_ERR_ARG ("Catalog has invalid sumw == 0"), as the reference raises.  Positions from
 * ra/dec then come from tc_generate_xyz(_device).  Host arrays for tc_catalog_finish
 * (copied to the device and back), device arrays for tc_catalog_finish_device (cols is a
 * host array of device pointers). */
#define TC_CAT_MAXCOLS 24
typedef struct {
    int64_t nkeep;           /* rows left */
    int64_t nobj;            /* rows with w != 0 (Catalog.nobj) */
    double sumw;             /* Catalog.sumw */
    int nontrivial_w;        /* Catalog.nontrivial_w */
    int64_t wpos_zero;       /* rows with wpos == 0 */
    int64_t wpos_conflicts;  /* of those, rows whose w was not 0 (the reference's logged error) */
    int64_t nan_counts[TC_CAT_MAXCOLS + 2];   /* NaNs per column, then w, then wpos */
} tc_catalog_info;
int tc_catalog_finish(int64_t n, int ncols, double* const* cols, double* w, double* wpos,
                      const int64_t* flag, int64_t ignore_flag, int w_given,
                      int keep_zero_weight, tc_catalog_info* info);
int tc_catalog_finish_device(int64_t n, int ncols, double* const* cols, double* w,
                             double* wpos, const int64_t* flag, int64_t ignore_flag,
                             int w_given, int keep_zero_weight, tc_catalog_info* info);

/* Catalog._get_center_size (treecorr/catalog.py:1330-1341; used by the triviallyZero tests
 * of the patch loops, treecorr/corr2base.py:776-800): out = (mean x, mean y, mean z, size),
 * the unweighted mean position and the largest distance of a point from it; z NULL for flat
 * catalogs (mean z = 0).  Host arrays for tc_catalog_center_size, device arrays for
 * tc_catalog_center_size_device.  n must be positive. */
int tc_catalog_center_size(int64_t n, const double* x, const double* y, const double* z,
                           double* out);
int tc_catalog_center_size_device(int64_t n, const double* x, const double* y,
                                  const double* z, double* out);

/* Self-check of the tcgen05 tensor-core path (no reference counterpart): one CTA computes
 * c[128 x n] = a[128 x k] * b[n x k]^T in TF32 through TMEM (k in 8..64, multiple of 8;
 * n in 16..64, multiple of 16).  Host arrays, row-major. */
int tc_tcgen05_selftest(const float* a, const float* b, float* c, int n, int k);

/* ---- Learned opening criterion (no reference counterpart) ----------------------------
 * A 5-64-64-1 ReLU network (FP32 master parameters, tc_mlp_nparam() floats: W1[64][5],
 * b1[64], W2[64][64], b2[64], w3[64], b3) revisits the cell pairs the bin_slop rule
 * (include/BinType.h:93-151) would split, when (s1+s2)^2 <= a^2 r^2 and
 * (s1+s2)^2 <= (cand_factor * b)^2 r^2 with min_sep <= r < max_sep: it accepts such a pair
 * into the bin of its separation when its output (a predicted log10 of the weight fraction
 * that would land in another bin) is <= threshold.  Inference runs in the traversal with
 * FP16 weights and FP32 accumulation.  Features: the larger and smaller cell size over
 * r * bin_size, the distance of log r to the nearest bin edge (in bin sizes), the position
 * of log r in the binned range, bin_size. */
int tc_mlp_nparam(void);

/* Enable (params != NULL) or disable the criterion for the following process calls. */
int tc_corr2_set_learned(tc_corr2* corr, const float* params, double threshold,
                         double cand_factor);

/* Training pairs: runs processAuto with the bin_slop rule (adding into the corr outputs as
 * usual) and samples about 1 in sample_mod of the candidate pairs; each sample gets the
 * features and the target log10(leak + 1e-5) from a point-by-point recount (pairs with
 * more than max_point_pairs point pairs get target NaN).  feat_out: max_samples x 5,
 * target_out: max_samples; *n_out = samples written. */
int tc_learn_collect(tc_corr2* corr, tc_field* field, int metric, int sample_mod,
                     int64_t max_samples, int64_t max_point_pairs, float* feat_out,
                     float* target_out, int64_t* n_out);

/* Mean-squared-error gradient of the network over n samples (FP32, on the device). */
int tc_mlp_grad(const float* params, const float* x, const float* y, int64_t n, float* grad,
                float* loss);

/* The traversal's network evaluation (FP16 mma) over n feature rows. */
int tc_mlp_infer(const float* params, const float* x, int64_t n, float* y);

/* Adam training on the device: steps mini-batches of `batch` samples; params in/out;
 * loss_out (may be NULL) receives the loss of every step. */
int tc_mlp_train(float* params, const float* x, const float* y, int64_t n, int steps,
                 int batch, float lr, unsigned seed, float* loss_out);

/* SetOMPThreads / GetOMPThreads (src/Corr2.cpp:995-1011).  The GPU path has no host
 * threads to set: both return 1, which the Python layer accepts. */
int tc_set_omp_threads(int num_threads);
int tc_get_omp_threads(void);

/* Fixed-order 2-point expansion (no reference counterpart; the reference's results repeat
 * bit for bit with num_threads = 1, tests/test_gg.py:573-574).  On (the default): the
 * children and tiles of every expansion launch are joined in warp order, so every warp
 * takes the same items in every run and all floating-point sums of a process call repeat
 * bit for bit.  Off: they are appended in the order warps finish (slightly faster; sums
 * then vary in the last bits from run to run).  Applies to the bin_slop and learned
 * criteria of process/processAuto/processCross (not to the patch batch or the
 * allocation-free call).  Returns the previous setting. */
int tc_set_deterministic(int on);
int tc_get_deterministic(void);

/* The 2-point expansion's level buffers (about 1 GB each at 10M points) come from the
 * current device's stream-ordered memory pool, which keeps them after a corr is freed so
 * that the next corr reuses them without driver calls.  tc_trim_memory returns the pool's
 * unused memory to the driver (no reference counterpart). */
int tc_trim_memory(void);

/* Message of the last failure on the calling thread ("" if none). */
const char* tc_last_error(void);

/* Number of CUDA kernels the library has launched since it was loaded (no reference
 * counterpart; used by benchmarks to report the device work behind a measurement). */
long long tc_launch_count(void);

/* The CUDA stream (cudaStream_t) on which the library launches its work, created on first
 * use; callers may record events on it to time the device work (no reference counterpart). */
void* tc_stream(void);

#ifdef __cplusplus
}
#endif

#endif /* TCGPU_H */
