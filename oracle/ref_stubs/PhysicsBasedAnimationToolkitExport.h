// Stand-in for the reference build's generated export header.
#define PBAT_API
