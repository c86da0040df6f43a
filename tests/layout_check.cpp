// Host-side check of the device index arithmetic (citcomcu_gb300/csrc/level.h):
// colour-major positions are a bijection on the nodes of a level, every
// stencil coefficient index is inside the 243*npad array and unique, and the
// gather of a row (the address pattern of row_dot in kernels.cu) stays inside
// the array for every node, row and neighbour slot.  Compiled and run by
// tests/test_layout.py with g++ (no GPU).
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../citcomcu_gb300/csrc/level.h"

static Lvl make(int ex, int ey, int ez)
{
	Lvl L = {};
	L.nox = ex + 1; L.noy = ey + 1; L.noz = ez + 1;
	L.elx = ex; L.ely = ey; L.elz = ez;
	L.nno = L.nox * L.noy * L.noz; L.nel = ex * ey * ez; L.neq = 3 * L.nno;
	L.npad = (L.nno + 31) / 32 * 32;
	const int N[3] = {L.nox, L.noy, L.noz};
	for(int a = 0; a < 3; ++a)
		for(int p = 0; p < 2; ++p)
			L.cnt[a][p] = (N[a] - p + 1) / 2;
	cg_set_offsets(L);
	return L;
}

static int fail(const char *m, int a, int b)
{
	printf("FAIL %s %d %d\n", m, a, b);
	return 1;
}

int main()
{
	const int sizes[][3] = {{4, 4, 4}, {8, 12, 8}, {16, 16, 16}, {2, 3, 2}, {4, 4, 2}, {8, 8, 4}, {1, 1, 1}, {32, 32, 32}};
	for(int aos = 0; aos < 2; ++aos)
	for(auto &sz : sizes)
	{
		Lvl L = make(sz[0], sz[1], sz[2]);
		L.aos = aos;
		if(L.coff[8] != L.nno)
			return fail("colour counts", L.coff[8], L.nno);
		std::vector<int> seen(L.nno, 0);
		for(int c = 0; c < 8; ++c)
			for(int q = 0; q < L.coff[c + 1] - L.coff[c]; ++q)
			{
				int x, y, z;
				cg_decode(L, c, q, x, y, z);
				if(x < 0 || x >= L.nox || y < 0 || y >= L.noy || z < 0 || z >= L.noz)
					return fail("decode range", c, q);
				if(cg_colour(x, y, z) != c || cg_pos(L, x, y, z) != L.coff[c] + q)
					return fail("pos inverse", c, q);
				seen[cg_node(L, x, y, z)]++;
			}
		for(int n = 0; n < L.nno; ++n)
			if(seen[n] != 1)
				return fail("bijection", n, seen[n]);
		std::vector<unsigned char> used(cg_kwords(L), 0);
		for(int p = 0; p < L.nno; ++p)
			for(int s = 0; s < 27; ++s)
				for(int i = 0; i < 3; ++i)
					for(int j = 0; j < 3; ++j)
					{
						const size_t k = cg_kidx(L, s, i, j, p);
						if(k >= cg_kwords(L))
							return fail("kidx range", p, s);
						if(used[k]++)
							return fail("kidx unique", p, s);
						// tiled: a tile is CG_TILE consecutive positions of one colour, the
						// lane of node ln reads tile word ((3s + j) * CG_TILE + ln) * 3 + i;
						// node-by-node kc = K + 243p + s, loads kc + 27(3i + j)
						int c = 0;
						while(p >= L.coff[c + 1])
							++c;
						const int q = p - L.coff[c];
						const size_t expect = aos ? (size_t)243 * p + s + 27 * (3 * i + j)
						                          : (size_t)(L.toff[c] + q / CG_TILE) * 243 * CG_TILE +
						                                ((3 * s + j) * CG_TILE + q % CG_TILE) * 3 + i;
						if(expect != k)
							return fail("gather pattern", p, s);
					}
		// BI[3p + i] inside 3*npad; vectors 3n + i inside neq
		if(3 * (size_t)(L.nno - 1) + 2 >= 3 * (size_t)L.npad)
			return fail("BI range", L.nno, L.npad);
		// local element nodes and their inverse
		for(int a = 0; a < 8; ++a)
			if(cg_local_index(cg_loc(a, 0), cg_loc(a, 1), cg_loc(a, 2)) != a)
				return fail("local index", a, 0);
	}
	// chunked ownership: every position has exactly the owner whose chunk
	// holds it, and the neighbour window of the cubes the 64^3 multigrid uses
	// (16 ranks): 5^3 -> 7, 9^3 -> 4, 17^3 -> 2, 33^3 -> 1
	const int cube[4][2] = {{4, 7}, {8, 4}, {16, 2}, {32, 1}};
	for(auto &cw : cube)
	{
		Lvl L = make(cw[0], cw[0], cw[0]);
		for(int y = 0; y < L.noy; ++y)
			for(int x = 0; x < L.nox; ++x)
				for(int z = 0; z < L.noz; ++z)
				{
					const int c = cg_colour(x, y, z), nc = L.coff[c + 1] - L.coff[c];
					const int q = cg_pos(L, x, y, z) - L.coff[c], r = cg_owner(L, x, y, z, 16);
					if(!(nc * r / 16 <= q && q < nc * (r + 1) / 16))
						return fail("owner chunk", q, r);
				}
		if(cg_owner_window(L, 16) != cw[1])
			return fail("owner window", cw[0], cg_owner_window(L, 16));
	}
	printf("OK\n");
	return 0;
}
