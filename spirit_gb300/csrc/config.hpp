// Reader of the reference's input-file format (core/docs/Input.md).  Keyword lookup follows
// core/src/io/Filter_File_Handle.cpp:124-160: the first non-comment line that begins with the
// keyword (case-insensitive prefix) wins, its remaining tokens are the values.
#pragma once
#include <sstream>
#include <string>
#include <vector>

namespace sg
{

class ConfigFile
{
public:
    bool load( const std::string & path );
    bool empty() const
    {
        return lines_.empty();
    }
    // positions the reader after `key` on its line; false if absent
    bool find( const std::string & key );
    // next line (after the last find/next_line), tokens readable with >>
    bool next_line();
    template<typename T>
    bool read( T & v )
    {
        return static_cast<bool>( iss_ >> v );
    }
    template<typename T>
    bool get( const std::string & key, T & v )
    {
        if( !find( key ) )
            return false;
        T tmp;
        if( iss_ >> tmp )
        {
            v = tmp;
            return true;
        }
        return false;
    }
    template<typename T>
    bool get3( const std::string & key, T * v )
    {
        if( !find( key ) )
            return false;
        T tmp[3];
        for( int i = 0; i < 3; ++i )
            if( !( iss_ >> tmp[i] ) )
                return false;
        for( int i = 0; i < 3; ++i )
            v[i] = tmp[i];
        return true;
    }

private:
    std::vector<std::string> lines_;
    size_t cursor_ = 0;
    std::istringstream iss_;
};

} // namespace sg
