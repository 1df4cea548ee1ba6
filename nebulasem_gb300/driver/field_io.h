/*
 * The euler app's field files `<name><index>.bin|.txt` (MeshField::read /
 * write, src/field/field.h:1409-1677, through the binary stream of
 * src/util/util.h:191-258: strings as a one-byte length and the bytes,
 * `Int` as uint32, values as raw little-endian doubles).
 *
 *   size <components> internal <count> { <values or initialisers> }
 *   boundary <n> { <patch> { type <NAME> ... } ... }
 *
 * A count of at most 4 lists initialiser expressions evaluated at the node
 * coordinates (uniform, cosine, cosine2, gaussian, linear, hydrostatic;
 * field.h:1421-1510); a larger count lists the interior values.  The
 * reference reads `.bin` before `.txt` (field.h:1579-1585) and writes
 * Controls::write_format (BINARY unless `write_format TEXT`), values with 12
 * significant digits in text.
 */
#ifndef NSEM_DRIVER_FIELD_IO_H
#define NSEM_DRIVER_FIELD_IO_H

#include <array>
#include <string>
#include <vector>

namespace nsem_driver {

struct BoundaryCond {
    std::string patch, type;
    std::vector<std::string> options;   /* keys other than `type` (not supported) */
};

struct Field {
    int ncomp = 1;
    std::vector<double> values;          /* interior nodes x ncomp */
    std::vector<BoundaryCond> bcs;
    const BoundaryCond* bc(const std::string& patch) const;
};

/* Read `<base>.bin` or `<base>.txt`.  cC: node coordinates (3 per node) of
 * the n_int interior nodes, gravity for the hydrostatic initialiser.  Throws
 * std::runtime_error; `found` is false (and nothing thrown) when neither file
 * exists. */
Field read_field(const std::string& base, int ncomp, const double* cC, long n_int,
                 const std::array<double, 3>& gravity, bool& found);

/* Write `<base>.bin` (binary) or `<base>.txt` */
void write_field(const std::string& base, const Field& f, bool binary);

}  // namespace nsem_driver

#endif
