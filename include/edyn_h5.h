/* HDF5 files in the layout of the output files (edyn_output_open, ...)
 * without a solver context: writing step groups of float64 rows, and
 * reading groups, datasets and attributes back. No GPU and no HDF5 library
 * is involved; the functions serve tools and checks around the reference's
 * results files (SRC/write_hdf5.f90, SRC/read_hdf5.f90, the post-processing
 * scripts' h5py reads).
 *
 * Return codes are those of edyn_gpu.h (EDYN_OK, EDYN_E_ARG, EDYN_E_IO);
 * edyn_h5_error() describes the calling thread's last failure. */
#ifndef EDYN_H5_H
#define EDYN_H5_H

#ifdef __cplusplus
extern "C" {
#endif

/* Creates (truncates) path; *h is the handle of the open file. */
int edyn_h5_create(const char* path, void** h);

/* Appends a group below the root group: nrow float64 datasets of n values,
 * rows[r * n .. r * n + n) named row_names[r], and nattr one-element
 * attributes (attr_is_int[a] != 0: int32, else float64). */
int edyn_h5_add_group(void* h, const char* name, int nattr, const char* const* attr_names, const int* attr_is_int,
                      const double* attr_values, int nrow, const char* const* row_names, const double* rows,
                      long long n);

/* Closes the file and frees the handle. */
int edyn_h5_close(void* h);

/* Members of a group ("" or "/" for the root) in its index (name) order,
 * each followed by '\n', groups marked by a trailing '/'. */
int edyn_h5_list(const char* path, const char* group, char* buf, long long len);

/* A dataset's values as doubles (*n of them; at most cap written). */
int edyn_h5_read(const char* path, const char* dataset, double* out, long long cap, long long* n);

/* An attribute's numeric values as doubles, or its text (fixed-length
 * strings) into buf when buf is not NULL. */
int edyn_h5_attr(const char* path, const char* object, const char* name, double* out, long long cap, long long* n,
                 char* buf, long long len);

/* The attribute names of an object, each followed by '\n'. */
int edyn_h5_attr_names(const char* path, const char* object, char* buf, long long len);

/* The step group name write_hdf5_b gives output nout at time time_total:
 * Fortran's ("nout",i6.6,"_time",e11.5) (SRC/write_hdf5.f90:168). */
int edyn_h5_step_name(int nout, double time, char* buf, int len);

const char* edyn_h5_error(void);

#ifdef __cplusplus
}
#endif

#endif
