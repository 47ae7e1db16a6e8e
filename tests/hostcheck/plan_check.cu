// Host-side checks of the FFT radix planner (radix_plan) and of the fast-division constants
// (make_fastdiv) used by the device kernels.  Built with nvcc as host code by tests/test_host_math.py;
// prints one line per failure and "ok" at the end.
#include "fft.cuh"

#include <cstdio>

using namespace sg;

static int failures = 0;

static void fail( const char * what, long long a, long long b )
{
    if( failures++ < 20 )
        std::printf( "FAIL %s %lld %lld\n", what, a, b );
}

// the division the device performs with the constants of make_fastdiv
static unsigned int host_fdiv( unsigned int n, const FastDiv & f )
{
    const unsigned int hi = (unsigned int)( ( (unsigned long long)n * f.m ) >> 32 );
    return ( hi + n ) >> f.l;
}

int main()
{
    // radix plans: every length up to the largest FFT extent
    const int supported[] = { 2, 3, 4, 5, 6, 7, 8, 9, 10, 12 };
    for( int L = 2; L <= MAX_FFT_LEN; ++L )
    {
        RadixPlan P;
        radix_plan( L, P );
        long long prod = 1;
        int ns = 0;
        for( int s = 0; s < 12 && P.radix[s] > 0; ++s, ++ns )
        {
            const int r = P.radix[s];
            bool prime = r >= 11; // direct-sum stages: prime factors above 7 only
            for( int p = 2; p * p <= r; ++p )
                prime = prime && r % p != 0;
            bool ok = prime;
            for( int q : supported )
                ok = ok || r == q;
            if( !ok )
                fail( "radix", L, r );
            if( P.div_lr[s].d != (unsigned)( L / r ) || P.div_ns[s].d != (unsigned)prod )
                fail( "stage divisors", L, s );
            prod *= r;
        }
        if( prod != L )
            fail( "product", L, prod );
        // 7-smooth lengths use register radices only, in at most ceil(log_12 L) + 2 stages
        int m = L;
        for( int p : { 2, 3, 5, 7 } )
            while( m % p == 0 )
                m /= p;
        if( m == 1 )
        {
            int minst = 0;
            for( long long t = 1; t < L; t *= 12 )
                ++minst;
            if( ns > minst + 2 )
                fail( "stages", L, ns );
        }
    }
    // known plans of the padded extents the tests and the ensemble use
    const int known[][5] = { { 360, 9, 8, 5, 0 }, { 84, 12, 7, 0, 0 }, { 80, 10, 8, 0, 0 }, { 54, 9, 6, 0, 0 },
                             { 12, 12, 0, 0, 0 } };
    for( const auto & k : known )
    {
        RadixPlan P;
        radix_plan( k[0], P );
        for( int s = 0; s < 4; ++s )
            if( P.radix[s] != k[s + 1] )
                fail( "known plan", k[0], s );
    }
    // fast division: exhaustive small divisors and dividends near multiples, and large ones
    for( unsigned int d = 1; d <= 4096; ++d )
    {
        const FastDiv f = make_fastdiv( d );
        for( unsigned int n = 0; n < 3 * d + 70000; n += ( n < 70000 ? 1 : d ) )
            if( host_fdiv( n, f ) != n / d )
                fail( "fdiv", d, n );
        for( unsigned int k = 1; k < 64; ++k )
        {
            const unsigned long long q = ( ( 1ull << 31 ) - 1 ) / d / k * k;
            for( long long dn = -1; dn <= 1; ++dn )
            {
                const long long n = (long long)( q * d ) + dn;
                if( n >= 0 && n < ( 1ll << 31 ) && host_fdiv( (unsigned)n, f ) != (unsigned)n / d )
                    fail( "fdiv large", d, n );
            }
        }
    }
    for( unsigned int d : { 4097u, 65535u, 65536u, 65537u, 1000003u, ( 1u << 30 ) - 1, 1u << 30, ( 1u << 31 ) - 1 } )
    {
        const FastDiv f = make_fastdiv( d );
        for( unsigned int n : { 0u, 1u, d - 1, d, d + 1, 2 * d - 1, ( 1u << 31 ) - 1, ( 1u << 31 ) - 2 } )
            if( n < ( 1u << 31 ) && host_fdiv( n, f ) != n / d )
                fail( "fdiv edge", d, n );
    }
    std::printf( failures ? "failures %d\n" : "ok\n", failures );
    return failures ? 1 : 0;
}
