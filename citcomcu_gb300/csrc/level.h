// Per-level mesh description shared by the host driver and the kernels.
//
// Node numbering follows CitcomCU (Construct_arrays.c:78-81, 0-based here):
//   n = z + x*noz + y*noz*nox,   velocity equation 3n+d (x, y, z interleaved)
//   element e = ez + ex*elz + ey*elz*elx (pressure lives on elements)
// Operator coefficients (the assembled 27-block stencil, 1/diag) are stored
// "colour-major": nodes are grouped by the parity of (z, x, y) into 8
// colours, so that one Gauss-Seidel colour sweep streams a contiguous slice
// of every coefficient array.
#pragma once

#include <stddef.h>

#define CITCOM_MAX_LEVELS 12

struct Lvl
{
	int nox, noy, noz;
	int nno, nel, neq;
	int elx, ely, elz;
	int npad;        // nno rounded up to a multiple of 32 (length of the per-node arrays)
	int aos;         // 1: small level, stencil stored node by node (243 contiguous words per node, slot fastest);
	                 // 0: stencil stored by tiles of 16 positions of one colour
	int cnt[3][2];   // number of indices of parity p along axis (0 x, 1 y, 2 z)
	int coff[9];     // colour offsets in colour-major order
	int toff[9];     // first tile of each colour (tiles of CG_TILE positions, a colour's last one partial)
	double h[3];     // element edge lengths (uniform per axis); in the sphere dtheta, dphi (radians), dr
	double J;        // Jacobian determinant hx*hy*hz/8 (box only)
	int sphere;      // 1: regional spherical shell segment, x, y, z = theta, phi, r (Geometry=Rsphere)
	double org[3];   // coordinates of node (0, 0, 0): 0, 0, 0 in the box; theta_north, phi_west (radians), r_inner
	// L2 residency of the tile-major stencil (tile.cu): with l2hint set, the
	// bulk copies of the first l2keep per mille of each colour's tiles carry
	// the evict_last priority and the others evict_first, so that the share
	// of a level that fits in L2 stays there across its sweeps while the
	// rest streams through without displacing it; l2hint 0: no hint
	int l2hint, l2keep;
};


#ifdef __CUDACC__
#define CG_HD __host__ __device__ __forceinline__
#else
#define CG_HD inline
#endif

// Element geometry is the same for every element of the box, and for every
// element of one (theta, r) column of the sphere (the segment is invariant
// under rotation about the polar axis by multiples of dphi): index of the
// geometry table entry of element (ex, ., ez)
CG_HD int cg_col(const Lvl &L, int ex, int ez) { return L.sphere ? ex * L.elz + ez : 0; }

CG_HD int cg_colour(int x, int y, int z) { return (z & 1) | ((x & 1) << 1) | ((y & 1) << 2); }

CG_HD int cg_node(const Lvl &L, int x, int y, int z) { return z + L.noz * (x + L.nox * y); }

CG_HD int cg_pos(const Lvl &L, int x, int y, int z)
{
	const int c = cg_colour(x, y, z);
	return L.coff[c] + (z >> 1) + L.cnt[2][z & 1] * ((x >> 1) + L.cnt[0][x & 1] * (y >> 1));
}

CG_HD void cg_decode(const Lvl &L, int c, int q, int &x, int &y, int &z)
{
	const int nz = L.cnt[2][c & 1], nx = L.cnt[0][(c >> 1) & 1];
	z = 2 * (q % nz) + (c & 1);
	const int t = q / nz;
	x = 2 * (t % nx) + ((c >> 1) & 1);
	y = 2 * (t / nx) + ((c >> 2) & 1);
}

// velocity constraint bits of a node: free slip on every wall (the reference's
// free-slip top/bottom with reflecting sides) constrains exactly the dof
// normal to each wall; bit 0 x, bit 1 y, bit 2 z
CG_HD unsigned cg_vflag(const Lvl &L, int x, int y, int z)
{
	return (unsigned)(x == 0 || x == L.nox - 1) | ((unsigned)(y == 0 || y == L.noy - 1) << 1) |
	       ((unsigned)(z == 0 || z == L.noz - 1) << 2);
}

// local node a (0..7) of an element -> (x, y, z) offset; the same sign
// pattern orders the 2x2x2 Gauss points (element_definitions.h:139-222)
CG_HD int cg_loc(int a, int d)
{
	// a: 0 (0,0,0) 1 (1,0,0) 2 (1,1,0) 3 (0,1,0) 4 (0,0,1) 5 (1,0,1) 6 (1,1,1) 7 (0,1,1)
	return d == 0 ? (((a & 3) == 1) || ((a & 3) == 2)) : d == 1 ? ((a & 3) >= 2) : (a >= 4);
}

// Stencil coefficient (neighbour slot s = (dz+1) + 3(dx+1) + 9(dy+1), row i,
// column j) of the node at colour-major position p.  Large levels: tiles of
// CG_TILE consecutive positions of one colour, each tile one contiguous block
// of 243 * CG_TILE words ordered [s][j][node][i] -- one bulk copy brings a
// tile into shared memory, where the 32 lanes of a warp (32 nodes, one slot)
// read a word each without bank conflicts.  Small levels keep a node's 243
// words together with the slot fastest, so the 27 lanes of a warp that relax
// one node read 27 consecutive words per (row, column) entry.
#define CG_TILE 32
#define CG_TILE_WORDS (243 * CG_TILE)
CG_HD size_t cg_kidx(const Lvl &L, int s, int i, int j, int p)
{
	if(L.aos)
		return (size_t)243 * p + 27 * (3 * i + j) + s;
	int c = 0;
	for(int k = 1; k < 8; ++k)
		c += (p >= L.coff[k]);
	const int q = p - L.coff[c];
	return (size_t)(L.toff[c] + q / CG_TILE) * CG_TILE_WORDS + (size_t)((3 * s + j) * CG_TILE + q % CG_TILE) * 3 + i;
}

// words of the stencil storage of a level
CG_HD size_t cg_kwords(const Lvl &L)
{
	return L.aos ? (size_t)243 * L.npad : (size_t)L.toff[8] * CG_TILE_WORDS;
}

// colour offsets and tile offsets from the per-axis parity counts
CG_HD void cg_set_offsets(Lvl &L)
{
	L.coff[0] = 0;
	L.toff[0] = 0;
	for(int c = 0; c < 8; ++c)
	{
		const int n = L.cnt[2][c & 1] * L.cnt[0][(c >> 1) & 1] * L.cnt[1][(c >> 2) & 1];
		L.coff[c + 1] = L.coff[c] + n;
		L.toff[c + 1] = L.toff[c] + (n + CG_TILE - 1) / CG_TILE;
	}
}

// levels up to this many nodes keep the node-by-node layout and are smoothed
// by one CTA (warp per node)
#define CG_SMALL_LEVEL_NODES 1400

// Chunked ownership of the colour-major positions among `nranks` workers:
// worker r owns positions [n_c r / nranks, n_c (r+1) / nranks) (integer
// division) of every colour c, n_c the colour's size.
CG_HD int cg_owner(const Lvl &L, int x, int y, int z, int nranks)
{
	const int c = cg_colour(x, y, z), nc = L.coff[c + 1] - L.coff[c];
	const int q = cg_pos(L, x, y, z) - L.coff[c];
	int r = (int)((long)q * nranks / nc);
	while(r > 0 && nc * r / nranks > q)
		--r;
	while(r + 1 < nranks && nc * (r + 1) / nranks <= q)
		++r;
	return r;
}

// the largest rank distance between the owner of a node and the owner of one
// of its 27 neighbours (host only)
inline int cg_owner_window(const Lvl &L, int nranks)
{
	int w = 0;
	for(int y = 0; y < L.noy; ++y)
		for(int x = 0; x < L.nox; ++x)
			for(int z = 0; z < L.noz; ++z)
			{
				const int r = cg_owner(L, x, y, z, nranks);
				for(int dy = -1; dy <= 1; ++dy)
					for(int dx = -1; dx <= 1; ++dx)
						for(int dz = -1; dz <= 1; ++dz)
						{
							const int X = x + dx, Y = y + dy, Z = z + dz;
							if(X < 0 || Y < 0 || Z < 0 || X >= L.nox || Y >= L.noy || Z >= L.noz)
								continue;
							const int d = cg_owner(L, X, Y, Z, nranks) - r;
							w = d > w ? d : (-d > w ? -d : w);
						}
			}
	return w;
}

CG_HD int cg_local_index(int ox, int oy, int oz)
{
	// inverse of cg_loc
	const int base = oy ? (ox ? 2 : 3) : (ox ? 1 : 0);
	return base + 4 * oz;
}
