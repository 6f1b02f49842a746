/*
 * floatybits.h -- drop-in declarations of the reference's C++/floatybits.h
 * (floatybits.h:17-97): the same names, argument order and meaning.  The
 * bit-vector helpers run on the host; split4pd, split8pd and mixsplit2
 * slice on the GPU through mdg_split (reference-compatible mode, so the
 * slices equal the reference's bit for bit).  Implemented in dropin.cu.
 */
#ifndef MDG_DROPIN_FLOATYBITS_H
#define MDG_DROPIN_FLOATYBITS_H

#include <cmath>
#include <iostream>
#include <random>
#include <vector>
using namespace std;

int val_bits(vector<int> bits);
vector<int> expandfracbits(double fr);
vector<int> expandexpbits(int n);
vector<int> bitform(double x);
vector<int> random_double_bits(int signbit, int exponent, bool fixfirst = true);
double double_rep(vector<int> bits);
vector<double> random_pd(int expmin, int expmax, int p);
bool is_balanced(double x, double y, int threshold);
void balance(double &x, double &y, int threshold);
void balance4(vector<double> &x, int a, int b);
vector<double> split4(vector<int> bits);
vector<double> split4pd(vector<double> x, int p);
void balance8(vector<double> &x, int a, int b);
vector<double> split8(vector<int> bits);
vector<double> split8pd(vector<double> x, int p);
void mixbalance(vector<double> &x, int a, int b);
vector<double> mixsplit2(vector<double> x);

#endif
