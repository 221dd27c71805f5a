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
 * plot/cmp_ay.py -- reads. No libhdf5 is needed to write it. Status codes and
 * sayram_last_error() are those of sayram_gpu.h; no function needs a GPU.
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

#ifdef __cplusplus
}
#endif

#endif /* SAYRAM_H5_H */
