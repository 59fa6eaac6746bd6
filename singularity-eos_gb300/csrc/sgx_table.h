// Table residency: the sp5-lite reader, the load-time table derivation of
// SpinerEOSDependsRhoT, and the registry of device table images.
#pragma once

#include <cstdint>
#include <string>

namespace sgx {

// Loads /<matid>/dependsLogRhoLogT and /<matid>/coldCurve from an sp5-lite
// image, derives the load-time tables and uploads the image to the current
// device. *handle receives the device address of the table header.
int table_load_spiner(const char *path, int matid, bool reproducible, uint64_t *handle,
                      std::string &msg);
// Loads /<matid>/dependsLogRhoLogT, /<matid>/dependsLogRhoLogSie and
// /<matid>/coldCurve for SpinerEOSDependsRhoSie and uploads its image.
int table_load_spiner_sie(const char *path, int matid, bool reproducible, uint64_t *handle,
                          std::string &msg);
// Loads a Helmholtz electron free-energy table (the reference's ASCII
// helm_table.dat layout) and uploads the per-cell Hermite records.
int table_load_helm(const char *path, uint64_t *handle, std::string &msg);
int table_free(uint64_t handle, std::string &msg);
size_t table_bytes(uint64_t handle);
// Density nodes of a resident Spiner table (0 if unknown).
int table_nrho(uint64_t handle);
// Whether a resident SpinerEOSDependsRhoSie table carries the float-float
// cells of its rho-sie grid (every value inside the float range).
bool table_has_sie_cells(uint64_t handle);
// Whether a resident Spiner table carries the thermal-energy bin index.
bool table_has_thermal_index(uint64_t handle);
// Spiner: derived tables in the reference's DBLIST order; Helmholtz: node
// values and fields in its DBLIST order. Returns the count or -1.
long table_dump(uint64_t handle, double *out, long cap);

// Gruneisen::ComputeRhoMax (eos_gruneisen.hpp:231-329), without the 0.99
// safety factor.
double gruneisen_compute_rho_max(double s1, double s2, double s3, double rho0, int *err);

} // namespace sgx
