/*
 * polgraw_gb300_host.h -- host side of the drop-in search program
 * (gwsearch-gb300), exported by libpolgraw_gb300.so.
 *
 * It re-implements, in this project's own C, the set-up and sky loop of the
 * reference network search that surround job_core():
 *   handle_opts        search/network/src-cpu/init.c:28-281
 *   read_grid          init.c:287-321
 *   search_settings    settings.c:16-81
 *   detectors_settings settings.c:92-246
 *   init_arrays        init.c:326-457 (data, sig2, ephemerides)
 *   narrow_down_band / read_lines / lines_in_band / fraction_of_band_vetoed
 *                      settings.c:327-656
 *   rogcvir            settings.c:253-275
 *   add_signal         init.c:462-651
 *   set_search_range   init.c:656-804 (+ gridr, auxi.c:143-212)
 *   read_checkpoints   init.c:868-917
 *   search             jobcore.c:51-184 (state file, trigger append)
 *   main               main.c:37-155
 * with the same command-line options, input files, trigger-file layout and
 * state-file semantics.  Differences are listed in the function comments.
 */
#ifndef POLGRAW_GB300_HOST_H
#define POLGRAW_GB300_HOST_H

#include "polgraw_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pa_host pa_host;

/* Exit-code-like results of the host steps. */
enum {
  PA_HOST_OK = 0,
  PA_HOST_EXIT_SUCCESS = 100,  /* reference would exit(EXIT_SUCCESS) here */
  PA_HOST_EXIT_FAILURE = 101,  /* reference would exit(EXIT_FAILURE) here */
  PA_HOST_INTERRUPTED = 102    /* stopped by PA_HOST_STOP_AT_SKY (pa_host_search) */
};

/* handle_opts(): parses argv (getopt_long_only, same option table) plus the
 * GB300 options -precision {mixed|fp64}, -phase {f64|fixed|ff},
 * -sbatch <spindowns per launch>, -skybatch <sky points per batch>,
 * -device <ordinal>.  Returns NULL with *rc set on --help or bad input. */
pa_host *pa_host_create(int argc, char **argv, int *rc);

/* main.c:58-135: output directory, grid, settings, detectors, data,
 * band narrowing and line veto, rogcvir, injection or range, -getrange,
 * checkpoint.  Returns PA_HOST_OK, PA_HOST_EXIT_SUCCESS (nothing left to
 * do: -getrange, fully vetoed band, empty state file) or
 * PA_HOST_EXIT_FAILURE. */
int pa_host_setup(pa_host *h);

/* search() (jobcore.c:51-184) over the context: state file before each
 * sky point, locked append of the candidate buffer when it holds more than
 * nfft records and at the end of each hemisphere, state file emptied at the
 * end (main.c:142-147).  Returns PA_HOST_OK or PA_HOST_EXIT_FAILURE.
 * Fault injection: with the environment variable PA_HOST_STOP_AT_SKY=k it
 * stops like a crash after writing the state file of its k-th sky-point
 * batch (0-based): buffered candidates are dropped, the state file stays,
 * and it returns PA_HOST_INTERRUPTED (the program exits with status 3). */
int pa_host_search(pa_host *h, pa_ctx *ctx);

/* Runs the whole program (gwsearch-gb300 main). */
int pa_host_main(int argc, char **argv);

void pa_host_destroy(pa_host *h);

/* Accessors for tests and embedding callers. */
const pa_settings *pa_host_settings(const pa_host *h);
const pa_detector *pa_host_detectors(const pa_host *h, int *nifo);
const pa_range *pa_host_range(const pa_host *h);
void pa_host_core_opts(const pa_host *h, pa_opts *out);
void pa_host_config(const pa_host *h, pa_config *out);
const char *pa_host_detector_name(const pa_host *h, int i);

/* The coincidence program coincidences-gb300 (coincidences/src/
 * coincidences.c main and read_trigger_files, init.c handle_opts_coinc and
 * manage_grid_matrix) over the device coincidence step pa_coinc_*: same
 * options, directory scan, .coi output and stderr summary.  Returns the
 * process exit code. */
int pa_coinc_main(int argc, char **argv);

/* Input generation: the reduced Fisher matrix (row-major 4x4) that the grid
 * generator writes into grid.bin after the grid matrix
 * (gridgen/src/FisherRM.cpp:17-100, postrmf(xi); ephemeris scaling of
 * gridgen/src/ReadEphemeris.cpp:82-100), from the ephemeris files' contents:
 * rSSB and rDet, n x 3 doubles each (Earth w.r.t. the SSB and detector w.r.t.
 * the Earth's centre), epsm (the obliquity stored at the end of DetSSB.bin)
 * and the initial time xi (the grid generator's default 0.5).  Equal to the
 * grid generator's matrix bit for bit.  PA_ERR_ARG for n < 5. */
int pa_fisher_reduced(const double *rSSB, const double *rDet, long long n, double epsm, double xi,
                      double *fisher);

/* Input generation: the grid generator's lattice (gridgen/main.cpp:955-1166
 * with GridS2.cpp, DensityS1.cpp, GridS1.cpp and num.cpp), i.e. the
 * grid.bin of a data segment, from the same ephemeris contents as
 * pa_fisher_reduced (rSSB, rDet: n x 3 doubles; epsm from DetSSB.bin).
 * Equal to the grid generator's grid.bin bit for bit. */
typedef struct pa_gridgen_opts {
  double c0;           /* covering parameter, minimal match squared (-c; the
                          generator's -m m sets c0 = m*m printed with six
                          decimals, main.cpp:172-190) */
  double xi;           /* initial time (-i, default 0.5) */
  int nfft_exp;        /* log2 of the FFT length (-n) */
  int method;          /* 0 automatic (main.cpp:1578-1606), 1 the A4* lattice
                          S1, 2 the tilted cell S2 (-a) */
  int nalpha, nradius; /* bisection and deep-hole depths of S2 (-na, -nr;
                          defaults 35, 20) */
  const char *table;   /* the generator's table of S2 cells, dataS2.txt
                          (read from its working directory); NULL: none */
} pa_gridgen_opts;

typedef struct pa_gridgen_out {
  int fftpad;          /* log2(nfft) - ceil(log2(n)) + 1 */
  double M[16];        /* grid-generating matrix as grid.bin stores it */
  double fisher[16];   /* reduced Fisher matrix at xi */
  double Mn[16];       /* the matrix before the division by n */
  int method;          /* 1 or 2, as chosen */
  double alpha;        /* S2: the cell's tilt */
  int alpha_from_table;/* S2: the tilt came from the table */
  double density;      /* density of covering of the basis (printed by the
                          generator) */
} pa_gridgen_out;

/* Returns PA_OK, or PA_ERR_ARG for n < 5, n > nfft, c0 outside (0, 1) or an
 * unknown method.  S1: among lattice vectors of exactly equal length the
 * first in enumeration order is taken (the generator's std::sort leaves that
 * order unspecified).  The table is read, never written (the generator
 * appends newly computed cells to its copy). */
int pa_gridgen(const double *rSSB, const double *rDet, long long n, double epsm, const pa_gridgen_opts *opts,
               pa_gridgen_out *out);

/* Writes the 388-byte grid.bin: int fftpad, then M, fisher and Mn (16
 * doubles each, main.cpp:1042-1160). */
int pa_gridgen_write(const char *path, const pa_gridgen_out *out);

#ifdef __cplusplus
}
#endif
#endif
