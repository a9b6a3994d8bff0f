/*
 * gb300kf_fieldmap.h — magnetic field maps from text files into the fitter's
 * grid (host code, no GPU).
 *
 * Replaces the reference's map ingestion: BField::txt::fieldMapperXYZ and
 * fieldMapperRZ (src/Plugins/BFieldUtils.cpp:16-99), which read the points
 * and hand them to Acts::fieldMapperXYZ / fieldMapperRZ
 * (src/MagneticField/BFieldMapUtils.cpp:17-240) to build the interpolated
 * grid, as Options::readBField does for the driver
 * (src/Plugins/BFieldOptions.cpp:33-61).
 *
 * File format (the reference's): one grid point per line, "x y z bx by bz"
 * (XYZ) or "r z br bz" (RZ), whitespace separated; lines that are empty,
 * blank or start with '%' or '#' are skipped.  Points are listed with the
 * last coordinate running fastest (row = (ix * ny + iy) * nz + iz for XYZ,
 * ir * nz + iz for RZ), the order the reference's localToGlobalBin assumes.
 * Positions are multiplied by `length_unit` (mm per file unit) and field
 * values by `field_unit` (GeV/(e*mm) per file unit; 0.000299792458 for
 * tesla).  With `first_octant` (`first_quadrant`) the file holds x, y, z >= 0
 * (r, z >= 0) starting at 0 and the grid is mirrored to the negative side,
 * values copied unchanged, as the reference mirrors them.
 *
 * The reference's grid places the file's points at the lower edges of its
 * bins and sets the bins beyond the last point to zero, so the field falls
 * linearly to zero over one more grid step above the largest coordinate.
 * The result here keeps that: one zero plane is appended above the last
 * point of each axis, and the fit's trilinear lookup (kf_field_t) then
 * equals the reference's within [min, max + step].
 *
 * On success `field` describes the grid (kind KF_FIELD_GRID3D, counts,
 * extent, scale 1, grid NULL) and *grid_host points to host memory of
 * nz*ny*nx*4 floats laid out as kf_field_t.grid wants it; copy it to the
 * device, set field->grid, and release the host copy with kf_field_map_free.
 * Errors: KF_ERR_IO (file unreadable), KF_ERR_INVALID_ARGUMENT (a malformed
 * line, a point count that is not the product of the axis counts, a point
 * out of the stated order, an axis of fewer than two points), with
 * kf_last_error_string() naming the file and line.
 */
#ifndef GB300KF_FIELDMAP_H
#define GB300KF_FIELDMAP_H

#include "gb300kf.h"

#ifdef __cplusplus
extern "C" {
#endif

int32_t kf_field_map_read_xyz(const char *path, double length_unit, double field_unit,
                              int32_t first_octant, kf_field_t *field, float **grid_host);

/* An (r, z) map, resampled onto the Cartesian grid given by n_xyz, min_xyz
 * and max_xyz (points per axis and extent in mm; n_xyz NULL: x and y over
 * [-r_max, r_max] and z over the map's z range, at the map's r and z steps).
 * Each Cartesian point holds the reference's RZ field there: bilinear in
 * (r, z) between the map's points (zero above the last point as above),
 * then (br cos phi, br sin phi, bz) with phi = atan2(y, x) (phi = 0 on the
 * axis).  Between the Cartesian points the fit interpolates trilinearly in
 * x, y, z, which differs from the reference's (r, z) interpolation by the
 * second derivative of the field times the squared Cartesian step. */
int32_t kf_field_map_read_rz(const char *path, double length_unit, double field_unit,
                             int32_t first_quadrant, const int32_t *n_xyz, const double *min_xyz,
                             const double *max_xyz, kf_field_t *field, float **grid_host);

/* An (r, z) map as the reference interpolates it: the grid of the file's
 * (br, bz) points plus the zero row above the last point on each axis
 * (kind KF_FIELD_GRID_RZ, nx = r points, ny = 1, nz = z points), looked up
 * bilinearly in (r, z) at r = |(x, y)| and rotated by the position's azimuth,
 * (br cos phi, br sin phi, bz) with phi = 0 on the axis (fieldMapperRZ,
 * BFieldMapUtils.cpp:17-136).  Same file format and checks as
 * kf_field_map_read_rz; first_quadrant mirrors z. */
int32_t kf_field_map_read_rz_native(const char *path, double length_unit, double field_unit,
                                    int32_t first_quadrant, kf_field_t *field,
                                    float **grid_host);

void kf_field_map_free(float *grid_host);

#ifdef __cplusplus
}
#endif

#endif /* GB300KF_FIELDMAP_H */
