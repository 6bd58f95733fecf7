// Stand-in for the reference's missing GluonFields.cpp: defines the two
// imprint arrays that GluonField.h declares.  They are only read when
// gluon_field_fluctuations=1, which the parity checker never sets.
#include "GluonField.h"
double GluonField::ImprintArrayLHC[600][600];
double GluonField::ImprintArrayRHIC[600][600];
