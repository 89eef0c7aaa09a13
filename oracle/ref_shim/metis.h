/* Eleven-argument k-way partitioner prototype the reference calls. */
#pragma once
void METIS_PartGraphKway(int*, int*, int*, int*, int*, int*, int*, int*, int*, int*, int*);
