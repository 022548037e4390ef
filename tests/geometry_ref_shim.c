/* geometry_ref_shim.c -- host access to the oracle's element-geometry
 * functions for tests/geometry_selftest.cc (test infrastructure only).
 * The oracle keeps them file-static; this unit includes its source and
 * exports thin wrappers. */
#include "lulesh_oracle.c"

void geo_ref_shape(const double *x, const double *y, const double *z, double *b24,
                   double *det)
{
    double b[3][8];
    shape_derivs(x, y, z, b, det);
    memcpy(b24, b, sizeof b);
}

void geo_ref_normals(const double *x, const double *y, const double *z, double *pfx,
                     double *pfy, double *pfz)
{
    node_normals(pfx, pfy, pfz, x, y, z);
}

void geo_ref_volume_derivative(const double *x, const double *y, const double *z, double *dvdx,
                               double *dvdy, double *dvdz)
{
    volume_derivative(dvdx, dvdy, dvdz, x, y, z);
}

double geo_ref_volume(const double *x, const double *y, const double *z)
{
    return elem_volume(x, y, z);
}

double geo_ref_char_length(const double *x, const double *y, const double *z, double volume)
{
    return char_length(x, y, z, volume);
}

void geo_ref_monoq_gradients(orc_domain *d) { monoq_gradients(d); }
