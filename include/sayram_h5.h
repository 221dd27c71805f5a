/*
 * sayram_h5.h -- the run's output file, in the HDF5 layout the reference writes
 * (Sayram-2D source/main.cc:57-89, through HighFive and xtensor-io):
 *
 *   /alpha0   (nx)       cell-centre equatorial pitch angles in degrees      main.cc:62, 65
 *   /logEN    (ny)       cell-centre ln E - ln E0                            main.cc:63, 66
 *   /f/<k>    (nx, ny)   f after k * save_every_step steps, alpha-major      main.cc:74, 82
 *   /t        (nplots+1) linspace(0, T, nplots + 1)                          main.cc:87-89
 *
 * All datasets are little-endian IEEE binary64, contiguous, in the classic HDF5 format
 * (superblock version 0, symbol-table groups) that libhdf5 -- and so h5py and the reference's
 * plot/cmp_ay.py -- reads. No libhdf5 is needed to write it, nor to read the D table below.
 * Status codes and sayram_last_error() are those of sayram_gpu.h; no function needs a GPU.
 */
#ifndef SAYRAM_H5_H
#define SAYRAM_H5_H

#include "sayram_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sayram_h5_s* sayram_h5;

/* Creates (truncates) the file: HighFive::File(filename, HighFive::File::Overwrite), main.cc:57. */
int sayram_h5_create(const char* path, sayram_h5* out);

/* xt::dump(file, path, array, xt::dump_mode::overwrite) (main.cc:65-66, 74, 82, 89): writes a
 * rank-`rank` FP64 array of shape dims[0..rank) in C order at `path` ("/f/3"), creating the
 * groups on the way; writing a path again replaces that dataset. rank 0 is a scalar. */
int sayram_h5_write(sayram_h5 h, const char* path, const double* data, int rank, const long long* dims);

/* Writes the group structure and the superblock, closes the file and frees the handle (also on
 * error). The file is complete only after this returns SAYRAM_OK. */
int sayram_h5_close(sayram_h5 h);

/* ---- input: xt::load_hdf5 and the Albert_Young D table --------------------------------------
 * The reader takes the classic format that libhdf5 and h5py write by default: superblock
 * version 0/1, symbol-table groups, version-1 object headers, contiguous or compact storage of
 * IEEE binary32/binary64 in either byte order. Anything else (superblock 2/3, chunked or
 * compressed storage, other types) is refused with SAYRAM_ERR_IO and a message saying what. */

/* xt::load_hdf5<...>(file, path): dataset `path` as FP64 in C order. On SAYRAM_OK, *rank and
 * dims[0..*rank) hold its shape and *data a library allocation of prod(dims) doubles, released
 * with sayram_h5_free. A rank above max_rank is SAYRAM_ERR_ARG. */
int sayram_h5_read(const char* file, const char* path, int max_rank, int* rank, long long* dims, double** data);
void sayram_h5_free(void* p);

/* Albert_Young_IO::read_D (source/Cases/Albert_Young_IO.cc:17-36): /alpha0 (degrees), /E, and
 * /Daa, /Dap, /Dpp of shape (n_alpha0, n_E) from the D file (the reference's D/<dID>.h5) into
 * arrays the library allocates; pass the table to sayram_set_dtable / sayram_batch_set_dtable,
 * then release it with sayram_dtable_free. */
int sayram_dtable_load_h5(const char* file, sayram_dtable* out);
void sayram_dtable_free(sayram_dtable* t);

#ifdef __cplusplus
}
#endif

#endif /* SAYRAM_H5_H */
