#include "config.hpp"

#include <algorithm>
#include <cctype>
#include <fstream>

namespace sg
{

bool ConfigFile::load( const std::string & path )
{
    lines_.clear();
    std::ifstream f( path );
    if( !f.good() )
        return false;
    std::string line;
    while( std::getline( f, line ) )
    {
        auto h = line.find( '#' );
        if( h != std::string::npos )
            line = line.substr( 0, h );
        // skip blank lines, keep everything else verbatim
        if( line.find_first_not_of( " \t\r\n" ) == std::string::npos )
            continue;
        auto s = line.find_first_not_of( " \t" );
        lines_.push_back( line.substr( s ) );
    }
    return true;
}

bool ConfigFile::find( const std::string & key )
{
    std::string k = key;
    std::transform( k.begin(), k.end(), k.begin(), ::tolower );
    for( size_t i = 0; i < lines_.size(); ++i )
    {
        std::string l = lines_[i];
        std::transform( l.begin(), l.end(), l.begin(), ::tolower );
        if( l.compare( 0, k.size(), k ) == 0 )
        {
            iss_.clear();
            iss_.str( lines_[i].substr( k.size() ) );
            cursor_ = i;
            return true;
        }
    }
    return false;
}

bool ConfigFile::next_line()
{
    if( cursor_ + 1 >= lines_.size() )
        return false;
    ++cursor_;
    iss_.clear();
    iss_.str( lines_[cursor_] );
    return true;
}

} // namespace sg
