// Writes the spherical element-geometry tables of one level (geometry.cu,
// compiled here for the host) as raw doubles, for the CPU checks of
// tests/test_sphere_geometry.py.
// usage: geometry_dump elx ely elz theta0 phi0 r0 dtheta dphi dr out.bin
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../citcomcu_gb300/csrc/kernels.h"

int main(int argc, char **argv)
{
	if(argc != 11)
		return 2;
	Lvl L;
	memset(&L, 0, sizeof(L));
	L.elx = atoi(argv[1]);
	L.ely = atoi(argv[2]);
	L.elz = atoi(argv[3]);
	L.nox = L.elx + 1;
	L.noy = L.ely + 1;
	L.noz = L.elz + 1;
	L.sphere = 1;
	for(int d = 0; d < 3; ++d)
	{
		L.org[d] = atof(argv[4 + d]);
		L.h[d] = atof(argv[7 + d]);
	}
	std::vector<Geo> g(geo_count(L));
	geo_fill_sphere(L, g.data());
	FILE *f = fopen(argv[10], "wb");
	if(!f || fwrite(g.data(), sizeof(Geo), g.size(), f) != g.size())
		return 1;
	fclose(f);
	printf("%zu %zu\n", g.size(), sizeof(Geo) / sizeof(double));
	return 0;
}
