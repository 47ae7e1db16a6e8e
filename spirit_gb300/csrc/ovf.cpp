// OVF 2.0 reader and writer (see ovf.hpp).
#include "ovf.hpp"

#include <algorithm>
#include <cctype>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <stdexcept>

namespace sg
{

namespace
{

constexpr int COUNT_DIGITS = 6; // zero-padded segment count, rewritten in place when appending

std::string lower( std::string s )
{
    std::transform( s.begin(), s.end(), s.begin(), []( unsigned char c ) { return (char)std::tolower( c ); } );
    return s;
}

std::string trim( const std::string & s )
{
    size_t a = s.find_first_not_of( " \t\r\n" );
    if( a == std::string::npos )
        return "";
    size_t b = s.find_last_not_of( " \t\r\n" );
    return s.substr( a, b - a + 1 );
}

std::string fmt_double( double v )
{
    std::ostringstream o;
    o << std::setprecision( 17 ) << v;
    return o.str();
}

std::string segment_text( const OvfSegment & seg, int format )
{
    std::ostringstream h;
    h << "# Begin: Segment\n# Begin: Header\n#\n";
    h << "# Title: " << seg.title << "\n#\n";
    std::istringstream desc( seg.desc );
    std::string line;
    bool any = false;
    while( std::getline( desc, line ) )
    {
        h << "# Desc: " << line << "\n";
        any = true;
    }
    if( !any )
        h << "# Desc: \n";
    h << "#\n# valuedim: " << seg.valuedim << "   ## field dimensionality\n";
    h << "# valuelabels: " << seg.valuelabels << "\n";
    h << "# valueunits: " << seg.valueunits << "\n#\n";
    h << "## Fundamental mesh measurement unit. Treated as a label:\n";
    h << "# meshunit: " << seg.meshunit << "\n#\n";
    const char ax[3] = { 'x', 'y', 'z' };
    for( int e = 0; e < 3; ++e )
        h << "# " << ax[e] << "min: " << fmt_double( seg.bounds_min[e] ) << "\n";
    for( int e = 0; e < 3; ++e )
        h << "# " << ax[e] << "max: " << fmt_double( seg.bounds_max[e] ) << "\n";
    h << "#\n# meshtype: " << seg.meshtype << "\n";
    for( int e = 0; e < 3; ++e )
        h << "# " << ax[e] << "base: " << fmt_double( seg.base[e] ) << "\n";
    for( int e = 0; e < 3; ++e )
        h << "# " << ax[e] << "stepsize: " << fmt_double( seg.step[e] ) << "\n";
    for( int e = 0; e < 3; ++e )
        h << "# " << ax[e] << "nodes: " << seg.nodes[e] << "\n";
    h << "#\n# End: Header\n#\n";
    const char * type = format == OVF_BIN4 ? "Binary 4" : ( format == OVF_TEXT ? "Text" : ( format == OVF_CSV ? "CSV" : "Binary 8" ) );
    h << "# Begin: Data " << type << "\n";
    std::string out = h.str();
    const size_t n  = seg.data.size();
    if( format == OVF_BIN4 )
    {
        const float check = 1234567.0f;
        out.append( reinterpret_cast<const char *>( &check ), 4 );
        for( size_t i = 0; i < n; ++i )
        {
            const float v = (float)seg.data[i];
            out.append( reinterpret_cast<const char *>( &v ), 4 );
        }
        out += "\n";
    }
    else if( format == OVF_TEXT || format == OVF_CSV )
    {
        std::ostringstream d;
        d << std::setprecision( 17 );
        const int dim = std::max( 1, seg.valuedim );
        for( size_t i = 0; i < n; ++i )
        {
            d << seg.data[i];
            d << ( ( i + 1 ) % dim == 0 ? "\n" : ( format == OVF_CSV ? ", " : " " ) );
        }
        out += d.str();
    }
    else
    {
        const double check = 123456789012345.0;
        out.append( reinterpret_cast<const char *>( &check ), 8 );
        out.append( reinterpret_cast<const char *>( seg.data.data() ), n * 8 );
        out += "\n";
    }
    out += std::string( "# End: Data " ) + type + "\n# End: Segment\n";
    return out;
}

std::string read_all( const std::string & file )
{
    std::ifstream f( file, std::ios::binary );
    if( !f )
        throw std::runtime_error( "cannot open \"" + file + "\"" );
    std::ostringstream o;
    o << f.rdbuf();
    return o.str();
}

// positions of "# Begin: Segment" lines
std::vector<size_t> segment_starts( const std::string & s )
{
    std::vector<size_t> out;
    size_t p = 0;
    while( ( p = s.find( "# Begin: Segment", p ) ) != std::string::npos )
    {
        if( p == 0 || s[p - 1] == '\n' )
            out.push_back( p );
        p += 16;
    }
    return out;
}

} // namespace

void ovf_write( const std::string & file, const OvfSegment & seg, int format, bool append )
{
    const std::string body = segment_text( seg, format );
    std::string content;
    int count = 1;
    if( append )
    {
        std::ifstream test( file, std::ios::binary );
        if( test.good() )
        {
            content = read_all( file );
            count   = (int)segment_starts( content ).size() + 1;
        }
    }
    char cnt[32];
    std::snprintf( cnt, sizeof( cnt ), "%0*d", COUNT_DIGITS, count );
    if( content.empty() )
        content = std::string( "# OOMMF OVF 2.0\n#\n# Segment count: " ) + cnt + "\n#\n";
    else
    {
        // rewrite the count in place
        size_t p = lower( content ).find( "# segment count:" );
        if( p == std::string::npos )
            throw std::runtime_error( "\"" + file + "\" has no segment count" );
        size_t e = content.find( '\n', p );
        content.replace( p, e - p, std::string( "# Segment count: " ) + cnt );
    }
    content += body;
    std::ofstream f( file, std::ios::binary | std::ios::trunc );
    if( !f )
        throw std::runtime_error( "cannot write \"" + file + "\"" );
    f.write( content.data(), (std::streamsize)content.size() );
}

int ovf_count( const std::string & file )
{
    try
    {
        return (int)segment_starts( read_all( file ) ).size();
    }
    catch( ... )
    {
        return 0;
    }
}

OvfSegment ovf_read( const std::string & file, int index )
{
    const std::string s   = read_all( file );
    const auto starts     = segment_starts( s );
    if( index < 0 || index >= (int)starts.size() )
        throw std::runtime_error( "\"" + file + "\" has no segment " + std::to_string( index ) );
    OvfSegment seg;
    seg.desc.clear();
    size_t p = starts[index];
    std::string type;
    // header lines until "# Begin: Data ..."
    while( p < s.size() )
    {
        size_t e         = s.find( '\n', p );
        std::string line = s.substr( p, e == std::string::npos ? std::string::npos : e - p );
        p                = e == std::string::npos ? s.size() : e + 1;
        std::string l    = trim( line );
        if( l.rfind( "##", 0 ) == 0 || l.size() < 2 || l[0] != '#' )
            continue;
        std::string body = trim( l.substr( 1 ) );
        std::string lb   = lower( body );
        if( lb.rfind( "begin: data", 0 ) == 0 )
        {
            type = lower( trim( body.substr( 11 ) ) );
            break;
        }
        size_t c = body.find( ':' );
        if( c == std::string::npos )
            continue;
        std::string key = lower( trim( body.substr( 0, c ) ) );
        std::string val = body.substr( c + 1 );
        size_t cm       = val.find( "##" );
        if( cm != std::string::npos )
            val = val.substr( 0, cm );
        val = trim( val );
        const char ax[3] = { 'x', 'y', 'z' };
        if( key == "title" )
            seg.title = val;
        else if( key == "desc" )
            seg.desc += ( seg.desc.empty() ? "" : "\n" ) + val;
        else if( key == "valuedim" )
            seg.valuedim = std::stoi( val );
        else if( key == "valuelabels" )
            seg.valuelabels = val;
        else if( key == "valueunits" )
            seg.valueunits = val;
        else if( key == "meshunit" )
            seg.meshunit = val;
        else if( key == "meshtype" )
            seg.meshtype = val;
        else
            for( int d = 0; d < 3; ++d )
            {
                const std::string a( 1, ax[d] );
                if( key == a + "nodes" )
                    seg.nodes[d] = std::stoi( val );
                else if( key == a + "min" )
                    seg.bounds_min[d] = std::stod( val );
                else if( key == a + "max" )
                    seg.bounds_max[d] = std::stod( val );
                else if( key == a + "base" )
                    seg.base[d] = std::stod( val );
                else if( key == a + "stepsize" )
                    seg.step[d] = std::stod( val );
            }
    }
    if( type.empty() )
        throw std::runtime_error( "\"" + file + "\": segment " + std::to_string( index ) + " has no data" );
    const size_t n = (size_t)seg.valuedim * seg.nodes[0] * seg.nodes[1] * seg.nodes[2];
    seg.data.resize( n );
    if( type == "binary 8" || type == "binary 4" )
    {
        const size_t w = type == "binary 8" ? 8 : 4;
        if( p + w * ( n + 1 ) > s.size() )
            throw std::runtime_error( "\"" + file + "\": truncated binary data" );
        if( w == 8 )
        {
            double check;
            std::memcpy( &check, s.data() + p, 8 );
            if( check != 123456789012345.0 )
                throw std::runtime_error( "\"" + file + "\": wrong binary check value" );
            std::memcpy( seg.data.data(), s.data() + p + 8, n * 8 );
        }
        else
        {
            float check;
            std::memcpy( &check, s.data() + p, 4 );
            if( check != 1234567.0f )
                throw std::runtime_error( "\"" + file + "\": wrong binary check value" );
            for( size_t i = 0; i < n; ++i )
            {
                float v;
                std::memcpy( &v, s.data() + p + 4 * ( i + 1 ), 4 );
                seg.data[i] = v;
            }
        }
    }
    else
    {
        // text or CSV: whitespace / comma separated numbers until "# End: Data"
        size_t e = s.find( "# End: Data", p );
        std::string txt = s.substr( p, e == std::string::npos ? std::string::npos : e - p );
        std::replace( txt.begin(), txt.end(), ',', ' ' );
        std::istringstream in( txt );
        for( size_t i = 0; i < n; ++i )
            if( !( in >> seg.data[i] ) )
                throw std::runtime_error( "\"" + file + "\": too few values in the data block" );
    }
    return seg;
}

} // namespace sg
