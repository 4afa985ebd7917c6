

Bin/rtm.x:   lin7@cees-gpu   Fri Aug 14 13:19:41 2015
		n1=300
		o1=0
		d1=4
		n2=300
		o2=0
		d2=4
		sets next: in="/data/lin7/dlambda-layer.H@"
		data_format="xdr_float"
