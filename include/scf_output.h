/*
 * scf_output.h -- device-resident field output for SIMCOFlow on GB300.
 *
 * scf_write_vtr writes what PrintResultVTK (src/PrintResult.f90:328-391)
 * writes: a VTK XML RectilinearGrid (.vtr) whose node coordinates are the
 * cell centres -+ half the cell widths and whose cell data are the interior
 * values of FP64 fields rounded to Float32, i fastest
 * (WriteDataArrayVTK, src/PrintResult.f90:393-421).  The fields are read
 * where they live, normally in device memory (the projection context's
 * corrected velocities and pressure, its level set and volume fractions):
 * a kernel gathers the interior cells and rounds them to FP32, so only the
 * Float32 values cross to the host.  Two layouts of the same values:
 *  - scf_write_vtr: the arrays raw in an appended section, one UInt64 byte
 *    count before each (the compact form, 3/4 of the inline size);
 *  - scf_write_vtr_binary: VTKFortran's "BINARY" layout, the one
 *    PrintResultVTK asks for (a_vtk_file%initialize(format='BINARY'),
 *    src/PrintResult.f90:364; xml_writer_binary_local of
 *    src/VTKFortran/src/lib/vtk_fortran_vtk_file_xml_writer_binary_local.f90):
 *    each array inline, the base64 of its Int32 byte count followed by the
 *    data (encode_binary_dataarray), with VTKFortran's tag text and
 *    indentation, so that the file is byte for byte the reference's.  The
 *    base64 is encoded on the device.
 */
#ifndef SCF_OUTPUT_H
#define SCF_OUTPUT_H

#include <stdint.h>
#include "scf_projection.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct scf_vtr_field {
    const char *name;        /* DataArray Name (no '"', '<', '&')               */
    const double *data;      /* ghosted (0:I+1,0:J+1,0:K+1) FP64 field          */
    int32_t on_device;       /* 1: data is a device pointer on `device`;
                                0: a host pointer                            */
} scf_vtr_field;

typedef struct scf_vtr_stats {
    double  ms_convert;      /* device gather + FP32 rounding (CUDA events)     */
    double  ms_d2h;          /* Float32 values to the host                      */
    double  ms_write;        /* the file write                                  */
    double  ms_total;
    int64_t bytes_file;
    int32_t gpu_launches;
} scf_vtr_stats;

/* xc, dx (I values), yc, dy (J), zc, dz (K): host arrays of the cell centres
 * and widths along each axis (TGrid%x(:,1,1), TGrid%dx(:,1,1), ...).  The
 * node coordinates are Float32 of xc(i) - dx(i)/2, i = 1..I, and
 * xc(I) + dx(I)/2, as PrintResultVTK computes them.  Fields with
 * on_device = 1 must be on CUDA device `device`.  J and K are at most
 * 65535.  Returns SCF_ERR_BAD_ARG for a bad name or size or a file that
 * cannot be written.                                                      */
int scf_write_vtr(const char *path, int32_t imax, int32_t jmax, int32_t kmax, const double *xc,
                  const double *dx, const double *yc, const double *dy, const double *zc, const double *dz,
                  int32_t nfields, const scf_vtr_field *fields, int32_t device, scf_vtr_stats *stats);

/* The same snapshot in VTKFortran's inline base64 layout (above), the file
 * PrintResultVTK writes (src/PrintResult.f90:328-391).  Its byte counts are
 * Int32 as in VTKFortran, so I*J*K is at most 536,870,911; larger grids
 * return SCF_ERR_BAD_ARG.                                                  */
int scf_write_vtr_binary(const char *path, int32_t imax, int32_t jmax, int32_t kmax, const double *xc,
                         const double *dx, const double *yc, const double *dy, const double *zc, const double *dz,
                         int32_t nfields, const scf_vtr_field *fields, int32_t device, scf_vtr_stats *stats);

/* Device pointers (ghosted FP64, on the context's device) of the fields a
 * projection context holds: u, v, w, p as corrected by the last
 * scf_update_puvw (or staged TVar before it), and the staged PCell phiL,
 * vofL and vof.  They stay valid until the context is destroyed; any
 * output may be NULL.                                                      */
int scf_ctx_device_fields(scf_ctx *ctx, const double **u, const double **v, const double **w,
                          const double **p, const double **phil, const double **vofl, const double **vof);

#ifdef __cplusplus
}
#endif
#endif
