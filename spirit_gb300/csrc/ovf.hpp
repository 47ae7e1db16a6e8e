// OOMMF OVF 2.0 vector-field files (the format the reference reads and writes through its
// thirdparty ovf library, core/src/io/OVF_File.cpp): text, comma-separated text, and binary with
// 4- or 8-byte IEEE values.  Written here from the public OVF 2.0 description.
#pragma once
#include <array>
#include <string>
#include <vector>

namespace sg
{

enum OvfFormat : int
{
    OVF_BIN  = 0, // binary in the precision of the API scalar (8 bytes here)
    OVF_BIN4 = 1,
    OVF_BIN8 = 2,
    OVF_TEXT = 3,
    OVF_CSV  = 4
};

struct OvfSegment
{
    std::string title;
    std::string desc; // free text; the engine keeps its random-stream positions here
    int valuedim = 3;
    std::string valuelabels = "spin_x spin_y spin_z";
    std::string valueunits  = "none none none";
    std::string meshunit    = "nm";
    std::string meshtype    = "rectangular";
    std::array<int, 3> nodes{ 1, 1, 1 };
    std::array<double, 3> bounds_min{ 0, 0, 0 }, bounds_max{ 0, 0, 0 }, base{ 0, 0, 0 }, step{ 1, 1, 1 };
    std::vector<double> data; // valuedim values per node, node index fastest in x
};

// write one segment (append = false: new file with one segment; true: add a segment and update
// the segment count of an existing file, or create it)
void ovf_write( const std::string & file, const OvfSegment & seg, int format, bool append );
// number of segments of a file (0 if it cannot be read)
int ovf_count( const std::string & file );
// read segment `index` (throws on a malformed file or a missing segment)
OvfSegment ovf_read( const std::string & file, int index );

} // namespace sg
